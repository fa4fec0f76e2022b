"""The CPU oracle pinned against the reference: the C restatement (oracle/port) must
reproduce the golden fixtures that the AxiomR reference itself produced
(tests/golden/make_golden.py), and, where the reference builds here, match it directly."""
import platform

import numpy as np
import pytest

from axiomr_gb300 import workloads as W
from helpers import GOLDEN, SHADING_EXTREMES, assert_parity, golden_names, load_golden, same_bits, shading_extreme_scene

X86 = platform.machine() in ("x86_64", "AMD64")


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)




@pytest.mark.parametrize("name", golden_names())
def test_port_matches_reference_golden(port, name):
    scene, vp, bgra_in, depth_in, bgra, depth = load_golden(name)
    got = port.draw(scene, vp, bgra=bgra_in, depth=depth_in)
    d = assert_parity(got, (bgra, depth), f"port vs golden {name}")
    if X86:  # same libm as the fixtures: colour is bit-exact too
        assert d["color_max_lsb"] == 0


def test_port_clip_and_setup_golden(port):
    z = np.load(GOLDEN / "stages.npz")
    for k in range(z["clip_in"].shape[0]):
        out = port.clip_triangle(z["clip_in"][k])
        n = int(z["clip_n"][k])
        assert out.shape[0] == n
        assert same_bits(out, z["clip_out"][k, :n]), k
        rec, bf = port.triangle(z["clip_in"][k], 320, 200)
        assert same_bits(rec, z["setup_out"][k]), k
        assert bf == bool(z["setup_backface"][k])


def test_port_sample_golden(port):
    z = np.load(GOLDEN / "stages.npz")
    assert same_bits(port.sample(z["tex"], z["uv"]), z["samples"])


def test_port_camera_golden(port):
    z = np.load(GOLDEN / "stages.npz")
    for p, exp in zip(z["cam_params"], z["cam_out"]):
        cam = W.Camera(tuple(p[0:3]), tuple(p[3:6]), float(p[6]), float(p[7]), (0, 0, 1, 1))
        got = port.camera(cam)
        if X86:
            assert same_bits(got, exp)
        else:  # sin/cos/tan/acos come from the host libm: allow one ulp
            assert np.all(np.abs(bits(got).astype(np.int64) - bits(exp).astype(np.int64)) <= 1)


SCENES = [
    lambda: W.sphere_scene(width=200, height=160, lon=32, lat=16, tex_size=64, shader=W.SHADER_BLINN_PHONG),
    lambda: W.sphere_scene(width=160, height=160, lon=20, lat=10, tex_size=32, shader=W.SHADER_PBR),
    lambda: W.sphere_scene(width=130, height=70, lon=48, lat=24, tex_size=32, distance=1.2, shader=W.SHADER_PHONG),
    lambda: W.soup_scene(count=6000, width=250, height=130, seed=21, edge_min=0.5, edge_max=60.0),
    lambda: W.heightfield_scene(n=96, width=300, height=170, tex_size=64, shader=W.SHADER_FLAT),
]


@pytest.mark.parametrize("make", SCENES)
def test_port_equals_reference(ref, port, make):
    sc = make()
    r = ref.render(sc)
    p = port.render(sc)
    assert np.array_equal(r[2], p[2]), "camera matrices differ"
    assert_parity(p[:2], r[:2], sc.name)
    assert np.array_equal(p[0], r[0])


@pytest.mark.parametrize("name", sorted(SHADING_EXTREMES))
def test_port_equals_reference_shading_extremes(ref, port, name):
    sc = shading_extreme_scene(name)
    vp = port.camera(sc.camera)[2]
    p, r = port.draw(sc, vp), ref.draw(sc, vp)
    assert same_bits(p[1], r[1]) and np.array_equal(p[0], r[0])


def test_port_equals_reference_stages_random(ref, port):
    rng = np.random.default_rng(7)
    for _ in range(3000):
        v = rng.normal(size=(3, 18)).astype(np.float32)
        v[:, 17] = np.abs(v[:, 17]) * rng.choice([0.5, 1.0, 2.0]) + rng.choice([0.0, -0.5])
        assert same_bits(ref.clip_triangle(v), port.clip_triangle(v))
        a, b = ref.triangle(v, 1920, 1080), port.triangle(v, 1920, 1080)
        assert same_bits(a[0], b[0]) and a[1] == b[1]


def test_port_shaders_equal_reference(ref, port):
    rng = np.random.default_rng(3)
    mat = W.Material(W.noise_texture(16, seed=1), W.noise_texture(16, seed=2), W.noise_texture(16, seed=3),
                     W.noise_texture(16, seed=4), W.noise_texture(16, seed=5), 0.7)
    for kind in range(5):
        sh = W.Shader(kind, (0.3, -1.0, 0.2), (1.5, 1.0, 0.5))
        for _ in range(300):
            verts = rng.normal(size=(3, 14)).astype(np.float32)
            verts[:, 3:5] = rng.uniform(0, 1, size=(3, 2))
            bar = rng.dirichlet([1, 1, 1]).astype(np.float32)
            model = np.eye(4, dtype=np.float32)
            model[:3, :3] += rng.normal(scale=0.3, size=(3, 3)).astype(np.float32)
            args = (sh, mat, model.reshape(16), np.eye(4, dtype=np.float32).reshape(16),
                    np.array([0, 0, 3], np.float32), verts, bar)
            assert same_bits(ref.shade(*args), port.shade(*args))


def test_port_draw_into_existing_framebuffer_matches_reference(ref, port):
    sc = W.sphere_scene(width=120, height=90, lon=16, lat=8, tex_size=16)
    u = W.uniform(5, sc.width * sc.height).reshape(sc.height, sc.width)
    depth = (u * 2 - 1).astype(np.float32)
    bgra = W.noise_texture(sc.width, sc.height, seed=6)
    vp = port.camera(sc.camera)[2]
    assert_parity(port.draw(sc, vp, bgra=bgra, depth=depth), ref.draw(sc, vp, bgra=bgra, depth=depth), "prefilled")


# ---------------------------------------------------------------- mesh ingest
def _obj_goldens():
    from helpers import GOLDEN

    return sorted(p.stem[len("obj_"):] for p in GOLDEN.glob("obj_*.npz"))


@pytest.mark.parametrize("name", _obj_goldens())
def test_obj_ingest_port_matches_reference_fixture(port, name):
    """The port's de-duplication, triangulation and tangent frames against the reference's
    Mesh(path) on the same OBJ text (fixture made by tests/golden/make_golden.py)."""
    import objfile
    from helpers import GOLDEN

    z = np.load(GOLDEN / f"obj_{name}.npz")
    parsed = objfile.parse_obj(str(z["text"]))
    verts, faces = port.obj_ingest(parsed)
    assert verts.shape == z["vertices"].shape and faces.shape == z["faces"].shape
    assert same_bits(verts, z["vertices"])
    assert np.array_equal(faces, z["faces"])
    assert np.array_equal(parsed["groups"], z["groups"])


def test_obj_ingest_port_matches_reference_live(port, ref, tmp_path):
    import objfile

    for seed in range(10, 16):
        text = objfile.tricky_obj(seed)
        path = tmp_path / f"t{seed}.obj"
        path.write_text(text)
        rv, rf, rg = ref.obj_load(str(path))
        parsed = objfile.parse_obj(text)
        pv, pf = port.obj_ingest(parsed)
        assert same_bits(pv, rv) and np.array_equal(pf, rf)
        assert np.array_equal(parsed["groups"], rg)
