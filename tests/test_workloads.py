"""The seeded workloads have the sizes the configurations name and are deterministic."""
import numpy as np

from axiomr_gb300 import workloads as W


def test_sphere_counts():
    pos, uv, nrm, tan, bit, idx = W.uv_sphere(64, 32)
    assert pos.shape == (65 * 33, 3) and idx.shape == (3968, 3)
    assert np.allclose(np.linalg.norm(nrm, axis=1), 1, atol=1e-6)
    # counter-clockwise seen from outside: outward geometric normals
    a, b, c = pos[idx[:, 0]], pos[idx[:, 1]], pos[idx[:, 2]]
    assert (np.einsum("ij,ij->i", np.cross(b - a, c - a), a + b + c) > 0).all()


def test_heightfield_counts():
    pos, uv, nrm, tan, bit, idx = W.heightfield(64, seed=2)
    assert pos.shape == (64 * 64, 3) and idx.shape == (2 * 63 * 63, 3)
    assert abs(pos[:, 1]).max() <= 0.2 + 1e-6
    a, b, c = pos[idx[:, 0]], pos[idx[:, 1]], pos[idx[:, 2]]
    assert (np.cross(b - a, c - a)[:, 1] > 0).all()  # front-facing seen from +y
    assert 2 * 1023 * 1023 == 2_093_058


def test_soup_and_textures_deterministic():
    a = W.soup_scene(count=1000, width=400, height=300)
    b = W.soup_scene(count=1000, width=400, height=300)
    assert np.array_equal(a.mesh.positions, b.mesh.positions)
    assert a.mesh.num_faces == 1000
    t1, t2 = W.noise_texture(64, seed=3), W.noise_texture(64, seed=3)
    assert t1.shape == (64, 64, 4) and np.array_equal(t1, t2)
    assert not np.array_equal(t1, W.noise_texture(64, seed=4))


def test_batch_plan():
    plan = W.batch_plan(512, seed=5)
    assert len(plan) == 512
    assert all(8 <= d.lon <= 256 and d.lat == d.lon // 2 for d in plan)
    assert {(d.width, d.height) for d in plan} <= set(W.BATCH_RESOLUTIONS)
    assert all(0 <= d.texture < 8 for d in plan)
