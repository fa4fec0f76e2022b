// Device-side mesh ingest: the part of AxiomR's OBJ loader after text parsing, on the GPU.
//
// Mesh::parseModelFile (src/mesh.cpp:300-415) turns every face-line corner into a Vertex
// (position, uv or (0,0), normal or (0,0,0)), numbers distinct vertices in order of first
// appearance (std::unordered_map with Vertex::operator==, include/mesh.hpp:15-17: all eight
// floats compare equal, so +0 == -0 and a NaN never matches) and fans each polygon into
// triangles; Mesh::calculateTangentBitangent (src/mesh.cpp:222-298) then sums per-face
// tangents and bitangents per vertex in face order and orthonormalises them. Here:
//   corner_keys     one thread per corner: its eight floats
//   insert          open-addressing hash table of corner indices; a slot keeps the smallest
//                   corner index of its key (atomicMin), i.e. the key's first appearance
//   first_flags     a corner is a vertex's first appearance when its slot holds itself
//   scan            exclusive prefix sum of the flags: vertex numbers in appearance order
//   emit_vertices / fan_faces / face_frames / incidence + vertex_frames
// The per-vertex sums run in face order (each vertex's incident (face, corner) entries are
// sorted before summing), so every float is the reference's. The text itself is parsed on
// the host (the reference's parser, or any other that produces the same pools).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>

#include "api_internal.h"
#include "api_types.h"
#include "fmath.cuh"

using namespace axr;
using namespace axr_internal;

namespace {

constexpr int kBlock = 256;

struct Key {
    float4 a;  // position x, y, z, uv.x
    float4 b;  // uv.y, normal x, y, z
};

__device__ __forceinline__ bool key_nan(const Key& k) {
    return k.a.x != k.a.x || k.a.y != k.a.y || k.a.z != k.a.z || k.a.w != k.a.w || k.b.x != k.b.x ||
           k.b.y != k.b.y || k.b.z != k.b.z || k.b.w != k.b.w;
}

__device__ __forceinline__ bool key_eq(const Key& p, const Key& q) {
    return p.a.x == q.a.x && p.a.y == q.a.y && p.a.z == q.a.z && p.a.w == q.a.w && p.b.x == q.b.x &&
           p.b.y == q.b.y && p.b.z == q.b.z && p.b.w == q.b.w;
}

__device__ __forceinline__ uint32_t key_hash(const Key& k) {
    const float f[8] = {k.a.x, k.a.y, k.a.z, k.a.w, k.b.x, k.b.y, k.b.z, k.b.w};
    uint32_t h = 2166136261u;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const uint32_t b = f[i] == 0.0f ? 0u : __float_as_uint(f[i]);  // +0 and -0 alike
        h = (h ^ b) * 16777619u;
        h ^= h >> 15;
    }
    return h;
}

__global__ void corner_keys_kernel(const float* __restrict__ pos, const float* __restrict__ uv, uint32_t n_uv,
                                   const float* __restrict__ nrm, uint32_t n_nrm, const int* __restrict__ corners,
                                   uint32_t nc, Key* keys) {
    const uint32_t c = blockIdx.x * kBlock + threadIdx.x;
    if (c >= nc) return;
    const int v = corners[3 * (size_t)c], t = corners[3 * (size_t)c + 1], n = corners[3 * (size_t)c + 2];
    const bool tv = t >= 0 && (uint32_t)t < n_uv, nv = n >= 0 && (uint32_t)n < n_nrm;
    Key k;
    k.a = make_float4(pos[3 * (size_t)v], pos[3 * (size_t)v + 1], pos[3 * (size_t)v + 2], tv ? uv[2 * (size_t)t] : 0.0f);
    k.b = make_float4(tv ? uv[2 * (size_t)t + 1] : 0.0f, nv ? nrm[3 * (size_t)n] : 0.0f,
                      nv ? nrm[3 * (size_t)n + 1] : 0.0f, nv ? nrm[3 * (size_t)n + 2] : 0.0f);
    keys[c] = k;
}

// Slot of corner c's key (inserting c when the key is new); -1 for a key with a NaN, which
// never matches. Probing visits every slot at most once.
__device__ int probe(const Key* keys, int* table, uint32_t mask, uint32_t c, bool insert) {
    const Key k = keys[c];
    if (key_nan(k)) return -1;
    uint32_t slot = key_hash(k) & mask;
    for (uint32_t step = 0; step <= mask; ++step) {
        int cur = atomicAdd(&table[slot], 0);
        if (cur < 0) {
            if (!insert) return -1;  // cannot happen after the insert pass
            const int prev = atomicCAS(&table[slot], -1, (int)c);
            if (prev < 0) return (int)slot;
            cur = prev;
        }
        if (key_eq(keys[cur], k)) {
            if (insert) atomicMin(&table[slot], (int)c);
            return (int)slot;
        }
        slot = (slot + 1) & mask;
    }
    return -1;
}

__global__ void insert_kernel(const Key* keys, int* table, uint32_t mask, uint32_t nc) {
    const uint32_t c = blockIdx.x * kBlock + threadIdx.x;
    if (c < nc) probe(keys, table, mask, c, true);
}

// first[c] = 1 when corner c is its vertex's first appearance; rep[c] = that first corner.
__global__ void first_flags_kernel(const Key* keys, int* table, uint32_t mask, uint32_t nc, uint32_t* first,
                                   uint32_t* rep) {
    const uint32_t c = blockIdx.x * kBlock + threadIdx.x;
    if (c >= nc) return;
    const int slot = probe(keys, table, mask, c, false);
    const uint32_t r = slot < 0 ? c : (uint32_t)table[slot];
    rep[c] = r;
    first[c] = r == c ? 1u : 0u;
}

// ---- exclusive prefix sum (block scans + a scan of the block totals)
constexpr int kScanBlock = 1024;

__global__ void scan_block_kernel(uint32_t* data, uint32_t n, uint32_t* block_sums) {
    __shared__ uint32_t warp_sums[kScanBlock / 32];
    const uint32_t i = blockIdx.x * kScanBlock + threadIdx.x;
    const uint32_t x = i < n ? data[i] : 0u;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t incl = x;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
        if (lane >= o) incl += y;
    }
    if (lane == 31) warp_sums[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        uint32_t s = lane < kScanBlock / 32 ? warp_sums[lane] : 0u;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, s, o);
            if (lane >= o) s += y;
        }
        if (lane < kScanBlock / 32) warp_sums[lane] = s;  // inclusive over warps
    }
    __syncthreads();
    const uint32_t before = (warp > 0 ? warp_sums[warp - 1] : 0u) + incl - x;
    if (i < n) data[i] = before;
    if (threadIdx.x == kScanBlock - 1 && block_sums) block_sums[blockIdx.x] = warp_sums[kScanBlock / 32 - 1];
}

__global__ void scan_add_kernel(uint32_t* data, uint32_t n, const uint32_t* block_offsets) {
    const uint32_t i = blockIdx.x * kScanBlock + threadIdx.x;
    if (i < n) data[i] += block_offsets[blockIdx.x];
}

cudaError_t scan_exclusive(uint32_t* data, uint32_t n, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    const uint32_t blocks = (n + kScanBlock - 1) / kScanBlock;
    if (blocks == 1) {
        scan_block_kernel<<<1, kScanBlock, 0, st>>>(data, n, nullptr);
        return cudaGetLastError();
    }
    uint32_t* sums = nullptr;
    cudaError_t e = cudaMallocAsync(&sums, sizeof(uint32_t) * blocks, st);
    if (e != cudaSuccess) return e;
    scan_block_kernel<<<blocks, kScanBlock, 0, st>>>(data, n, sums);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = scan_exclusive(sums, blocks, st);
    if (e == cudaSuccess) {
        scan_add_kernel<<<blocks, kScanBlock, 0, st>>>(data, n, sums);
        e = cudaGetLastError();
    }
    cudaFreeAsync(sums, st);
    return e;
}

// first corners -> vertex arrays (position, uv, normal); every corner -> its vertex number
__global__ void emit_vertices_kernel(const Key* keys, const uint32_t* first, const uint32_t* prefix,
                                     const uint32_t* rep, uint32_t nc, float4* pos, float2* uv, float4* nrm,
                                     uint32_t* vid) {
    const uint32_t c = blockIdx.x * kBlock + threadIdx.x;
    if (c >= nc) return;
    vid[c] = prefix[rep[c]];
    if (!first[c]) return;
    const Key k = keys[c];
    const uint32_t v = prefix[c];
    pos[v] = make_float4(k.a.x, k.a.y, k.a.z, 0.0f);
    uv[v] = make_float2(k.a.w, k.b.x);
    nrm[v] = make_float4(k.b.y, k.b.z, k.b.w, 0.0f);
}

// polygon p (corner offset, face offset from the host) -> its fan (c0, ci, ci+1)
__global__ void fan_faces_kernel(const uint32_t* vid, const uint32_t* poly_corner, const uint32_t* poly_face,
                                 const uint32_t* poly_size, uint32_t np, uint32_t* idx) {
    const uint32_t p = blockIdx.x * kBlock + threadIdx.x;
    if (p >= np) return;
    const uint32_t n = poly_size[p], o = poly_corner[p], f0 = poly_face[p];
    for (uint32_t i = 1; i + 1 < n; ++i) {
        uint32_t* f = idx + 3 * (size_t)(f0 + i - 1);
        f[0] = vid[o];
        f[1] = vid[o + i];
        f[2] = vid[o + i + 1];
    }
}

// per-face tangent and bitangent (src/mesh.cpp:226-257), and each corner's incidence count
__global__ void face_frames_kernel(const uint32_t* idx, uint32_t nf, const float4* pos, const float2* uv,
                                   const float4* nrm, float4* ft, float4* fb, uint32_t* count) {
    const uint32_t f = blockIdx.x * kBlock + threadIdx.x;
    if (f >= nf) return;
    const uint32_t i0 = idx[3 * (size_t)f], i1 = idx[3 * (size_t)f + 1], i2 = idx[3 * (size_t)f + 2];
    const float4 p0 = pos[i0], p1 = pos[i1], p2 = pos[i2];
    const f3 e1 = sub(mk3(p1.x, p1.y, p1.z), mk3(p0.x, p0.y, p0.z));
    const f3 e2 = sub(mk3(p2.x, p2.y, p2.z), mk3(p0.x, p0.y, p0.z));
    const float2 u0 = uv[i0], u1 = uv[i1], u2 = uv[i2];
    const float d1x = fsub(u1.x, u0.x), d1y = fsub(u1.y, u0.y), d2x = fsub(u2.x, u0.x), d2y = fsub(u2.y, u0.y);
    const float den = fsub(fmul(d1x, d2y), fmul(d2x, d1y));
    const float4 n0v = nrm[i0];
    const f3 n0 = mk3(n0v.x, n0v.y, n0v.z);
    f3 t, b;
    if (fabsf(den) < 1e-8f) {
        t = fabsf(n0.x) > 0.8f ? mk3(0.0f, 1.0f, 0.0f) : mk3(1.0f, 0.0f, 0.0f);
        b = cross(n0, t);
    } else {
        const float r = frcp(den);
        t = mul(r, sub(mul(d2y, e1), mul(d1y, e2)));
        b = mul(r, add(mul(-d2x, e1), mul(d1x, e2)));
        if (dot(cross(n0, t), b) < 0.0f) b = neg(b);
    }
    ft[f] = make_float4(t.x, t.y, t.z, 0.0f);
    fb[f] = make_float4(b.x, b.y, b.z, 0.0f);
    atomicAdd(&count[i0], 1u);
    atomicAdd(&count[i1], 1u);
    atomicAdd(&count[i2], 1u);
}

// incidence lists: entry f*3+k of face f's corner k in its vertex's list (unordered)
__global__ void incidence_kernel(const uint32_t* idx, uint32_t nf, const uint32_t* offset, uint32_t* cursor,
                                 uint32_t* entries) {
    const uint32_t f = blockIdx.x * kBlock + threadIdx.x;
    if (f >= nf) return;
    for (int k = 0; k < 3; ++k) {
        const uint32_t v = idx[3 * (size_t)f + k];
        entries[offset[v] + atomicAdd(&cursor[v], 1u)] = 3u * f + (uint32_t)k;
    }
}

// per vertex: its entries sorted (face order), the sums, then the orthonormal frame
// (src/mesh.cpp:260-297; the reference's two fallbacks test glm's vec3::length(), which is
// the component count 3, and never run)
__global__ void vertex_frames_kernel(uint32_t nv, const uint32_t* offset, const uint32_t* count, uint32_t* entries,
                                     const float4* ft, const float4* fb, const float4* nrm, float4* tan, float4* bit) {
    const uint32_t v = blockIdx.x * kBlock + threadIdx.x;
    if (v >= nv) return;
    uint32_t* e = entries + offset[v];
    const uint32_t n = count[v];
    for (uint32_t i = 1; i < n; ++i) {  // insertion sort: lists are short
        const uint32_t x = e[i];
        uint32_t j = i;
        while (j > 0 && e[j - 1] > x) {
            e[j] = e[j - 1];
            --j;
        }
        e[j] = x;
    }
    f3 ts = mk3(0.0f, 0.0f, 0.0f), bs = mk3(0.0f, 0.0f, 0.0f);
    for (uint32_t i = 0; i < n; ++i) {
        const uint32_t f = e[i] / 3u;
        const float4 a = ft[f], b = fb[f];
        ts = add(ts, mk3(a.x, a.y, a.z));
        bs = add(bs, mk3(b.x, b.y, b.z));
    }
    const float4 nv4 = nrm[v];
    const f3 nn = mk3(nv4.x, nv4.y, nv4.z);
    f3 t = n > 0 ? ts : mk3(1.0f, 0.0f, 0.0f);
    t = sub(t, mul(nn, dot(nn, t)));
    t = normalize(t);
    f3 b = cross(nn, t);
    const float hand = dot(bs, b) < 0.0f ? -1.0f : 1.0f;
    b = mul(b, hand);
    tan[v] = make_float4(t.x, t.y, t.z, 0.0f);
    bit[v] = make_float4(b.x, b.y, b.z, 0.0f);
}

unsigned grid(size_t n) { return (unsigned)std::max<size_t>(1, (n + kBlock - 1) / kBlock); }

}  // namespace

extern "C" axr_status axr_mesh_create_from_obj(axr_context* ctx, const axr_obj_desc* d, axr_mesh** out) {
    NvtxRange nvtx_range("axr_mesh_create_from_obj");
    if (!ctx || !d || !out) return fail(ctx, AXR_E_INVALID, "NULL argument");
    *out = nullptr;
    if ((d->num_positions && !d->positions) || (d->num_uvs && !d->uvs) || (d->num_normals && !d->normals) ||
        (d->num_corners && !d->corners) || (d->num_polygons && !d->polygon_sizes) ||
        (d->num_groups && !d->groups) || (d->num_materials && !d->materials))
        return fail(ctx, AXR_E_INVALID, "OBJ descriptor arrays missing");
    // host side: polygon offsets (corners and faces), checks
    const uint32_t nc = d->num_corners, np = d->num_polygons;
    std::vector<uint32_t> poly_corner(np), poly_face(np);
    uint64_t corners = 0, faces = 0;
    for (uint32_t p = 0; p < np; ++p) {
        poly_corner[p] = (uint32_t)corners;
        poly_face[p] = (uint32_t)faces;
        corners += d->polygon_sizes[p];
        if (d->polygon_sizes[p] >= 3) faces += d->polygon_sizes[p] - 2;
    }
    if (corners != nc) return fail(ctx, AXR_E_INVALID, "polygon sizes add up to %llu corners, not %u",
                                   (unsigned long long)corners, nc);
    if (faces > kMaxOrdinal + 1ull) return fail(ctx, AXR_E_CAPACITY, "a draw is limited to %u faces", kMaxOrdinal + 1u);
    for (uint64_t i = 0; i < nc; ++i)
        if (d->corners[3 * i] < 0 || (uint32_t)d->corners[3 * i] >= d->num_positions)
            return fail(ctx, AXR_E_INVALID, "corner %llu names position %d of %u", (unsigned long long)i,
                        d->corners[3 * i], d->num_positions);
    const uint32_t nf = (uint32_t)faces;
    uint64_t drawn = 0;
    for (uint32_t g = 0; g < d->num_groups; ++g) {
        if ((uint64_t)d->groups[g].start_face + d->groups[g].face_count > nf)
            return fail(ctx, AXR_E_INVALID, "group %u covers faces beyond the mesh", g);
        if (d->groups[g].material >= d->num_materials)
            return fail(ctx, AXR_E_INVALID, "group %u names material %u of %u", g, d->groups[g].material,
                        d->num_materials);
        drawn += d->groups[g].face_count;
    }
    std::lock_guard<std::mutex> lk(ctx->mu);
    DeviceGuard g(ctx->device);
    cudaStream_t st = ctx->stream;
    uint32_t cap = 16;
    while (cap < 2u * std::max<uint32_t>(nc, 1u)) cap <<= 1;

    // device inputs and scratch
    float *dpos = nullptr, *duv = nullptr, *dnrm = nullptr;
    int* dcorners = nullptr;
    uint32_t *dpc = nullptr, *dpf = nullptr, *dps = nullptr;
    Key* keys = nullptr;
    int* table = nullptr;
    uint32_t *first = nullptr, *prefix = nullptr, *rep = nullptr, *vid = nullptr;
    cudaError_t e = cudaSuccess;
    auto alloc = [&](auto** p, size_t bytes) {
        if (e == cudaSuccess) e = cudaMallocAsync(reinterpret_cast<void**>(p), std::max<size_t>(bytes, 16), st);
    };
    auto put = [&](void* dst, const void* src, size_t bytes) {
        if (e == cudaSuccess && bytes) e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st);
    };
    alloc(&dpos, 12ull * d->num_positions);
    alloc(&duv, 8ull * d->num_uvs);
    alloc(&dnrm, 12ull * d->num_normals);
    alloc(&dcorners, 12ull * nc);
    alloc(&dpc, 4ull * np);
    alloc(&dpf, 4ull * np);
    alloc(&dps, 4ull * np);
    alloc(&keys, sizeof(Key) * nc);
    alloc(&table, 4ull * cap);
    alloc(&first, 4ull * nc);
    alloc(&prefix, 4ull * nc);
    alloc(&rep, 4ull * nc);
    alloc(&vid, 4ull * nc);
    put(dpos, d->positions, 12ull * d->num_positions);
    put(duv, d->uvs, 8ull * d->num_uvs);
    put(dnrm, d->normals, 12ull * d->num_normals);
    put(dcorners, d->corners, 12ull * nc);
    put(dpc, poly_corner.data(), 4ull * np);
    put(dpf, poly_face.data(), 4ull * np);
    put(dps, d->polygon_sizes, 4ull * np);
    if (e == cudaSuccess) e = cudaMemsetAsync(table, 0xFF, 4ull * cap, st);
    if (e == cudaSuccess && nc) {
        corner_keys_kernel<<<grid(nc), kBlock, 0, st>>>(dpos, duv, d->num_uvs, dnrm, d->num_normals, dcorners, nc, keys);
        insert_kernel<<<grid(nc), kBlock, 0, st>>>(keys, table, cap - 1, nc);
        first_flags_kernel<<<grid(nc), kBlock, 0, st>>>(keys, table, cap - 1, nc, first, rep);
        e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaMemcpyAsync(prefix, first, 4ull * nc, cudaMemcpyDeviceToDevice, st);
        if (e == cudaSuccess) e = scan_exclusive(prefix, nc, st);
        ctx->launches += 3;
    }
    // vertex count = prefix[nc-1] + first[nc-1]
    uint32_t nv = 0;
    if (e == cudaSuccess && nc) {
        uint32_t last[2] = {0, 0};
        e = cudaMemcpyAsync(&last[0], prefix + nc - 1, 4, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(&last[1], first + nc - 1, 4, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        nv = last[0] + last[1];
    }
    auto* m = new axr_mesh();
    m->device = ctx->device;
    m->num_vertices = nv;
    m->num_faces = nf;
    m->num_groups = d->num_groups;
    m->num_materials = d->num_materials;
    if (e == cudaSuccess) e = dmalloc(&m->pos, nv);
    if (e == cudaSuccess) e = dmalloc(&m->nrm, nv);
    if (e == cudaSuccess) e = dmalloc(&m->tan, nv);
    if (e == cudaSuccess) e = dmalloc(&m->bit, nv);
    if (e == cudaSuccess) e = dmalloc(&m->uv, nv);
    if (e == cudaSuccess) e = dmalloc(&m->idx, 3ull * nf);
    if (e == cudaSuccess) e = dmalloc(&m->staging, 3ull * nv);
    if (e == cudaSuccess) e = dmalloc(&m->groups, std::max<uint32_t>(1, d->num_groups));
    if (e == cudaSuccess) e = dmalloc(&m->materials, std::max<uint32_t>(1, d->num_materials));
    float4 *ft = nullptr, *fb = nullptr;
    uint32_t *count = nullptr, *offset = nullptr, *cursor = nullptr, *entries = nullptr;
    alloc(&ft, 16ull * nf);
    alloc(&fb, 16ull * nf);
    alloc(&count, 4ull * nv);
    alloc(&offset, 4ull * nv);
    alloc(&cursor, 4ull * nv);
    alloc(&entries, 12ull * nf);
    if (e == cudaSuccess) e = cudaMemsetAsync(count, 0, 4ull * nv, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(cursor, 0, 4ull * nv, st);
    if (e == cudaSuccess && nc) {
        emit_vertices_kernel<<<grid(nc), kBlock, 0, st>>>(keys, first, prefix, rep, nc, m->pos, m->uv, m->nrm, vid);
        fan_faces_kernel<<<grid(np), kBlock, 0, st>>>(vid, dpc, dpf, dps, np, m->idx);
        e = cudaGetLastError();
        ctx->launches += 2;
    }
    if (e == cudaSuccess && nf) {
        face_frames_kernel<<<grid(nf), kBlock, 0, st>>>(m->idx, nf, m->pos, m->uv, m->nrm, ft, fb, count);
        e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaMemcpyAsync(offset, count, 4ull * nv, cudaMemcpyDeviceToDevice, st);
        if (e == cudaSuccess) e = scan_exclusive(offset, nv, st);
        if (e == cudaSuccess) {
            incidence_kernel<<<grid(nf), kBlock, 0, st>>>(m->idx, nf, offset, cursor, entries);
            e = cudaGetLastError();
        }
        ctx->launches += 2;
    }
    if (e == cudaSuccess && nv) {
        vertex_frames_kernel<<<grid(nv), kBlock, 0, st>>>(nv, offset, count, entries, ft, fb, m->nrm, m->tan, m->bit);
        e = cudaGetLastError();
        ctx->launches += 1;
    }
    // groups and materials as axr_mesh_create builds them
    std::vector<DevGroup> groups(std::max<uint32_t>(1, d->num_groups));
    uint32_t base = 0;
    for (uint32_t k = 0; k < d->num_groups; ++k) {
        groups[k] = DevGroup{d->groups[k].start_face, d->groups[k].face_count, base, d->groups[k].material};
        base += d->groups[k].face_count;
    }
    m->num_drawn = base;
    std::vector<DevMaterial> mats(std::max<uint32_t>(1, d->num_materials));
    for (uint32_t k = 0; k < d->num_materials; ++k) {
        const axr_material_desc& md = d->materials[k];
        DevMaterial& dm = mats[k];
        dm = DevMaterial{};
        auto view = [](const axr_texture* t) {
            DevTexture v{};
            if (t) {
                v.texels = t->texels;
                v.width = t->width;
                v.height = t->height;
            }
            return v;
        };
        dm.diffuse = view(md.diffuse);
        dm.bump = view(md.bump);
        dm.metallic = view(md.metallic);
        dm.roughness = view(md.roughness);
        dm.ao = view(md.ao);
        dm.specular_exponent = md.specular_exponent;
    }
    put(m->groups, groups.data(), sizeof(DevGroup) * groups.size());
    put(m->materials, mats.data(), sizeof(DevMaterial) * mats.size());
    // bounding sphere for batch planning: over the position pool (a superset of the vertices)
    mesh_bounds(d->positions, d->num_positions, m->bound_center, &m->bound_radius);
    void* temps[] = {dpos, duv, dnrm, dcorners, dpc, dpf, dps, keys, table, first, prefix, rep, vid,
                     ft, fb, count, offset, cursor, entries};
    for (void* p : temps)
        if (p) cudaFreeAsync(p, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        dfree(m->pos); dfree(m->nrm); dfree(m->tan); dfree(m->bit); dfree(m->uv); dfree(m->idx);
        dfree(m->staging); dfree(m->groups); dfree(m->materials);
        delete m;
        return cuda_fail(ctx, e, "mesh ingest");
    }
    (void)drawn;
    *out = m;
    return AXR_OK;
}

extern "C" axr_status axr_mesh_read(axr_context* ctx, const axr_mesh* m, float* vertices14, uint32_t* indices3) {
    if (!ctx || !m) return fail(ctx, AXR_E_INVALID, "NULL argument");
    std::lock_guard<std::mutex> lk(ctx->mu);
    DeviceGuard g(ctx->device);
    const uint32_t nv = m->num_vertices;
    std::vector<float4> pos(nv), nrm(nv), tan(nv), bit(nv);
    std::vector<float2> uv(nv);
    auto get = [&](void* dst, const void* src, size_t bytes) {
        if (src && bytes) AXR_CUDA(ctx, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, ctx->stream));
        return AXR_OK;
    };
    axr_status s = AXR_OK;
    if (vertices14) {
        if ((s = get(pos.data(), m->pos, 16ull * nv)) != AXR_OK) return s;
        if ((s = get(nrm.data(), m->nrm, 16ull * nv)) != AXR_OK) return s;
        if ((s = get(uv.data(), m->uv, 8ull * nv)) != AXR_OK) return s;
        if ((s = get(tan.data(), m->tan, 16ull * nv)) != AXR_OK) return s;
        if ((s = get(bit.data(), m->bit, 16ull * nv)) != AXR_OK) return s;
    }
    if (indices3 && (s = get(indices3, m->idx, 12ull * m->num_faces)) != AXR_OK) return s;
    AXR_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (vertices14)
        for (uint32_t i = 0; i < nv; ++i) {
            float* o = vertices14 + 14ull * i;
            const float f[14] = {pos[i].x, pos[i].y, pos[i].z, uv[i].x, uv[i].y, nrm[i].x, nrm[i].y, nrm[i].z,
                                 m->tan ? tan[i].x : 0.f, m->tan ? tan[i].y : 0.f, m->tan ? tan[i].z : 0.f,
                                 m->bit ? bit[i].x : 0.f, m->bit ? bit[i].y : 0.f, m->bit ? bit[i].z : 0.f};
            std::memcpy(o, f, sizeof(f));
        }
    return AXR_OK;
}

extern "C" axr_status axr_mesh_counts(const axr_mesh* m, uint32_t* vertices, uint32_t* faces, uint32_t* drawn) {
    if (!m) return fail(nullptr, AXR_E_INVALID, "mesh is NULL");
    if (vertices) *vertices = m->num_vertices;
    if (faces) *faces = m->num_faces;
    if (drawn) *drawn = m->num_drawn;
    return AXR_OK;
}
