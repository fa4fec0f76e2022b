/* Oracle test infrastructure: C restatement of AxiomR's mesh ingest after OBJ parsing:
 * the vertex de-duplication and fan triangulation of Mesh::parseModelFile
 * (src/mesh.cpp:300-415) and Mesh::calculateTangentBitangent (src/mesh.cpp:222-298).
 *
 * Input: the attribute pools ("v", "vt", "vn" lines) and, per face line, its corners as
 * (v, vt, vn) index triples, 0-based, with the corners whose position index is invalid
 * already dropped (the parser skips them, mesh.cpp:367). A corner's vertex is
 * (position, uv or (0,0), normal or (0,0,0)); two corners share a vertex when all eight
 * floats compare equal (Vertex::operator==, include/mesh.hpp:15-17; +0 and -0 compare and
 * hash equal, a NaN never matches), and vertices are numbered in order of first
 * appearance. A polygon of n corners becomes the fan (c0, ci, ci+1), i = 1..n-2. */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "axo_port.h"
#include "vmath.h"

typedef struct {
    float p[3], uv[2], n[3];
} corner_vertex;

static int has_nan(const corner_vertex* v) {
    for (int k = 0; k < 3; ++k)
        if (v->p[k] != v->p[k] || v->n[k] != v->n[k]) return 1;
    return v->uv[0] != v->uv[0] || v->uv[1] != v->uv[1];
}

static int same(const corner_vertex* a, const corner_vertex* b) {
    for (int k = 0; k < 3; ++k)
        if (!(a->p[k] == b->p[k]) || !(a->n[k] == b->n[k])) return 0;
    return a->uv[0] == b->uv[0] && a->uv[1] == b->uv[1];
}

static uint64_t hash_vertex(const corner_vertex* v) {
    const float* f = &v->p[0];
    uint64_t h = 1469598103934665603ull;
    for (int k = 0; k < 8; ++k) {
        float x = f[k] == 0.0f ? 0.0f : f[k]; /* +0 and -0 hash alike */
        uint32_t b;
        memcpy(&b, &x, 4);
        h = (h ^ b) * 1099511628211ull;
    }
    return h;
}

int port_obj_ingest(const axo_obj* in, float* verts_out, uint32_t* nv_out, uint32_t* faces_out, uint32_t* nf_out) {
    const uint32_t nc = in->num_corners;
    corner_vertex* cv = (corner_vertex*)malloc(sizeof(corner_vertex) * (nc ? nc : 1));
    uint32_t* vid = (uint32_t*)malloc(sizeof(uint32_t) * (nc ? nc : 1));
    uint32_t cap = 16;
    while (cap < 2 * nc) cap <<= 1;
    int64_t* table = (int64_t*)malloc(sizeof(int64_t) * cap); /* corner index of a vertex's first use */
    if (!cv || !vid || !table) return -1;
    for (uint32_t i = 0; i < cap; ++i) table[i] = -1;
    uint32_t nv = 0;
    for (uint32_t c = 0; c < nc; ++c) {
        const int32_t v = in->corners[3 * c], t = in->corners[3 * c + 1], n = in->corners[3 * c + 2];
        corner_vertex* x = &cv[c];
        for (int k = 0; k < 3; ++k) x->p[k] = in->positions[3 * (size_t)v + k];
        const int tv = t >= 0 && (uint32_t)t < in->num_uvs, nvld = n >= 0 && (uint32_t)n < in->num_normals;
        x->uv[0] = tv ? in->uvs[2 * (size_t)t] : 0.0f;
        x->uv[1] = tv ? in->uvs[2 * (size_t)t + 1] : 0.0f;
        for (int k = 0; k < 3; ++k) x->n[k] = nvld ? in->normals[3 * (size_t)n + k] : 0.0f;
        int64_t first = -1;
        uint64_t slot = 0;
        if (!has_nan(x)) {
            slot = hash_vertex(x) & (cap - 1);
            while (table[slot] >= 0) {
                if (same(&cv[table[slot]], x)) {
                    first = table[slot];
                    break;
                }
                slot = (slot + 1) & (cap - 1);
            }
        }
        if (first >= 0) {
            vid[c] = vid[first];
        } else {
            if (!has_nan(x)) table[slot] = c;
            vid[c] = nv;
            float* o = verts_out + 14 * (size_t)nv;
            memcpy(o, x->p, 12);
            memcpy(o + 3, x->uv, 8);
            memcpy(o + 5, x->n, 12);
            memset(o + 8, 0, 24);
            ++nv;
        }
    }
    /* fan triangulation */
    uint32_t nf = 0, at = 0;
    for (uint32_t p = 0; p < in->num_polygons; ++p) {
        const uint32_t n = in->polygon_sizes[p];
        for (uint32_t i = 1; i + 1 < n; ++i) {
            faces_out[3 * nf] = vid[at];
            faces_out[3 * nf + 1] = vid[at + i];
            faces_out[3 * nf + 2] = vid[at + i + 1];
            ++nf;
        }
        at += n;
    }
    /* tangents and bitangents (mesh.cpp:222-298): per-face vectors summed per vertex in
     * face order; a vertex no face uses keeps the defaults */
    v3* tacc = (v3*)calloc(nv ? nv : 1, sizeof(v3));
    v3* bacc = (v3*)calloc(nv ? nv : 1, sizeof(v3));
    unsigned char* used = (unsigned char*)calloc(nv ? nv : 1, 1);
    if (!tacc || !bacc || !used) return -1;
#define VP(i) V3(verts_out[14 * (size_t)(i)], verts_out[14 * (size_t)(i) + 1], verts_out[14 * (size_t)(i) + 2])
#define VUV(i) V2(verts_out[14 * (size_t)(i) + 3], verts_out[14 * (size_t)(i) + 4])
#define VN(i) V3(verts_out[14 * (size_t)(i) + 5], verts_out[14 * (size_t)(i) + 6], verts_out[14 * (size_t)(i) + 7])
    for (uint32_t f = 0; f < nf; ++f) {
        const uint32_t i0 = faces_out[3 * f], i1 = faces_out[3 * f + 1], i2 = faces_out[3 * f + 2];
        const v3 e1 = sub3(VP(i1), VP(i0)), e2 = sub3(VP(i2), VP(i0));
        const v2 uv0 = VUV(i0), uv1 = VUV(i1), uv2 = VUV(i2);
        const v2 d1 = V2(uv1.x - uv0.x, uv1.y - uv0.y), d2 = V2(uv2.x - uv0.x, uv2.y - uv0.y);
        const float den = d1.x * d2.y - d2.x * d1.y;
        v3 t, b;
        if (fabsf(den) < 1e-8f) {
            const v3 n0 = VN(i0);
            t = fabsf(n0.x) > 0.8f ? V3(0.0f, 1.0f, 0.0f) : V3(1.0f, 0.0f, 0.0f);
            b = cross3(n0, t);
        } else {
            const float r = 1.0f / den;
            t = smul3(r, sub3(smul3(d2.y, e1), smul3(d1.y, e2)));
            b = smul3(r, add3(smul3(-d2.x, e1), smul3(d1.x, e2)));
            const v3 expected = cross3(VN(i0), t);
            if (dot3(expected, b) < 0.0f) b = neg3(b);
        }
        const uint32_t ix[3] = {i0, i1, i2};
        for (int k = 0; k < 3; ++k) {
            tacc[ix[k]] = add3(tacc[ix[k]], t);
            bacc[ix[k]] = add3(bacc[ix[k]], b);
            used[ix[k]] = 1;
        }
    }
    for (uint32_t i = 0; i < nv; ++i) {
        const v3 n = VN(i);
        v3 t = used[i] ? tacc[i] : V3(1.0f, 0.0f, 0.0f);
        t = sub3(t, mul3s(n, dot3(n, t)));
        t = normalize3(t);
        v3 b = cross3(n, t);
        /* handedness against the accumulated bitangent (zero for an unused vertex) */
        const float hand = dot3(bacc[i], b) < 0.0f ? -1.0f : 1.0f;
        b = mul3s(b, hand);
        /* the reference's fallbacks test glm's vec3::length(), the component count 3, and
         * never run */
        float* o = verts_out + 14 * (size_t)i;
        o[8] = t.x; o[9] = t.y; o[10] = t.z;
        o[11] = b.x; o[12] = b.y; o[13] = b.z;
    }
#undef VP
#undef VUV
#undef VN
    free(cv);
    free(vid);
    free(table);
    free(tacc);
    free(bacc);
    free(used);
    *nv_out = nv;
    *nf_out = nf;
    return 0;
}
