"""OBJ text for the mesh-ingest tests: a writer for generated models and a parser that
reads text the way the reference's Mesh::parseModelFile does (src/mesh.cpp:300-415) up to
its vertex de-duplication: "v" / "vt" / "vn" pools, "usemtl" groups counted in
triangulated faces, and per "f" line the corners whose position index is valid, as
0-based (v, vt, vn) triples with vt / vn set to -1 when absent or not yet defined."""
from __future__ import annotations

import numpy as np


def fmt(x) -> str:
    """Shortest decimal that reads back as the same float32."""
    return np.format_float_positional(np.float32(x), unique=True, trim="-")


def parse_obj(text: str) -> dict:
    positions, uvs, normals = [], [], []
    corners, sizes, groups = [], [], []
    faces = 0
    group_start = 0
    for line in text.split("\n"):
        if not line:
            continue
        tok = line.split()
        if not tok:
            continue
        kind = tok[0]
        if kind == "v":
            positions.append([np.float32(float(t)) for t in tok[1:4]])
        elif kind == "vt":
            uvs.append([np.float32(float(t)) for t in tok[1:3]])
        elif kind == "vn":
            normals.append([np.float32(float(t)) for t in tok[1:4]])
        elif kind == "usemtl":
            if groups:
                groups[-1][1] = faces - group_start
            groups.append([faces, 0])
            group_start = faces
        elif kind == "f":
            poly = []
            for t in tok[1:]:
                parts = t.split("/")
                v = int(parts[0]) - 1 if parts and parts[0] else -1
                vt = int(parts[1]) - 1 if len(parts) > 1 and parts[1] else -1
                vn = int(parts[2]) - 1 if len(parts) > 2 and parts[2] else -1
                if v < 0 or v >= len(positions):
                    continue
                vt = vt if 0 <= vt < len(uvs) else -1
                vn = vn if 0 <= vn < len(normals) else -1
                poly.append((v, vt, vn))
            corners.extend(poly)
            sizes.append(len(poly))
            if len(poly) >= 3:
                faces += len(poly) - 2
        if groups:
            groups[-1][1] = faces - group_start
    return {
        "positions": np.asarray(positions, np.float32).reshape(-1, 3),
        "uvs": np.asarray(uvs, np.float32).reshape(-1, 2),
        "normals": np.asarray(normals, np.float32).reshape(-1, 3),
        "corners": np.asarray(corners, np.int32).reshape(-1, 3),
        "polygon_sizes": np.asarray(sizes, np.uint32),
        "groups": np.asarray(groups, np.uint64).reshape(-1, 2),
        "num_faces": faces,
    }


def write_obj(positions, uvs, normals, polygons, groups=()) -> str:
    """polygons: lists of (v, vt, vn) 0-based triples (vt / vn None to omit); groups:
    (polygon index, material name) pairs opening a usemtl group before that polygon."""
    out = []
    for p in positions:
        out.append("v " + " ".join(fmt(x) for x in p))
    for t in uvs:
        out.append("vt " + " ".join(fmt(x) for x in t))
    for n in normals:
        out.append("vn " + " ".join(fmt(x) for x in n))
    opens = dict(groups)
    for k, poly in enumerate(polygons):
        if k in opens:
            out.append(f"usemtl {opens[k]}")
        toks = []
        for v, vt, vn in poly:
            if vn is not None:
                toks.append(f"{v + 1}/{'' if vt is None else vt + 1}/{vn + 1}")
            elif vt is not None:
                toks.append(f"{v + 1}/{vt + 1}")
            else:
                toks.append(f"{v + 1}")
        out.append("f " + " ".join(toks))
    return "\n".join(out) + "\n"


def sphere_obj(lon: int = 24, lat: int = 12) -> str:
    """A UV sphere written with separate v / vt / vn pools (one entry per grid point), so
    the seam and pole corners share positions but not uvs: the de-duplication has work."""
    pos, uv, nrm, polys = [], [], [], []
    for i in range(lat + 1):
        th = np.pi * i / lat
        for j in range(lon + 1):
            ph = 2 * np.pi * j / lon
            p = (np.sin(th) * np.cos(ph), np.cos(th), np.sin(th) * np.sin(ph))
            pos.append(p)
            nrm.append(p)
            uv.append((j / lon, 1.0 - i / lat))
    for i in range(lat):
        for j in range(lon):
            a, b = i * (lon + 1) + j, (i + 1) * (lon + 1) + j
            polys.append([(a, a, a), (b, b, b), (b + 1, b + 1, b + 1), (a + 1, a + 1, a + 1)])  # quads
    return write_obj(pos, uv, nrm, polys, [(0, "body"), (len(polys) // 2, "lower")])


def tricky_obj(seed: int = 0) -> str:
    """Edge cases of the de-duplication and tangent generation: repeated attribute
    triples, +0 / -0, corners without vt or vn, pentagons and triangles,
    position indices past the pool (dropped corners), a vt index defined only later
    (absent at its face line), zero-area uv triangles (the fallback tangent), a face
    using one vertex twice, and vertices no face uses."""
    rng = np.random.default_rng(seed)
    pos = rng.uniform(-1, 1, (12, 3)).astype(np.float32)
    pos[3] = pos[2]                      # same position twice in the pool
    pos[5] = (0.0, -0.0, 0.5)
    pos[6] = (-0.0, 0.0, 0.5)            # equal to pos[5] under ==
    uv = rng.uniform(0, 1, (8, 2)).astype(np.float32)
    uv[4] = uv[5] = uv[6] = (0.25, 0.25)  # degenerate uv triangle
    nrm = rng.normal(size=(6, 3)).astype(np.float32)
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    nrm[0] = (0.9, 0.1, 0.0)              # |n.x| > 0.8 branch of the fallback
    nrm[5] = (0.0, -0.0, 1.0)
    lines = []
    lines += ["v " + " ".join(fmt(x) for x in p) for p in pos]
    lines += ["vt " + " ".join(fmt(x) for x in t) for t in uv[:7]]
    lines += ["vn " + " ".join(fmt(x) for x in n) for n in nrm]
    lines += [
        "usemtl a",
        "f 1/1/1 2/2/2 3/3/3",
        "f 3/3/3 4/3/3 2/2/2",              # 4 is 3 again: same vertex
        "f 1/5/1 2/6/1 5/7/1",              # zero-area uv: fallback tangent, |n.x| > 0.8
        "f 6/1/2 7/1/2 8/2/2 9/3/2 10/4/2",  # pentagon; 6 and 7 differ only in the sign of 0
        "f 1 2 8",                          # no vt, no vn
        "f 2//3 8//3 9//3",                 # no vt
        "usemtl b",
        "f 9/4/6 10/4/6 11/5/6",            # the same three vertices twice
        "f 9/4/6 10/4/6 11/5/6",
        "f 1/1/1 1/1/1 2/2/2",              # one vertex used twice by a face
        "f 1/8/1 2/8/1 3/2/1",              # vt 8 does not exist yet: uv (0,0)
        "f 40/1/1 2/1/1 3/1/1 4/2/2",       # position 40 does not exist: corner dropped
        "f 41 42",                          # nothing left: no face
        "f 12/7/4 11/6/5",                  # two corners: vertices that no face uses
    ]
    lines += ["vt " + " ".join(fmt(x) for x in uv[7])]
    lines += ["f 1/8/1 2/8/1 3/2/1"]           # now vt 8 exists
    return "\n".join(lines) + "\n"
