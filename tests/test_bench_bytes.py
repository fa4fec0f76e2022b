"""Host-side accounting of bench.py (no GPU): the algorithmic bytes behind the roofline
entries and the flat serving figures of the line."""
import sys
from pathlib import Path

import pytest

sys.path.insert(0, str(Path(__file__).resolve().parents[1]))
import bench  # noqa: E402
from axiomr_gb300 import workloads as W  # noqa: E402


def _scenes(widths):
    return [W.sphere_scene(width=w, height=32, lon=8, lat=4, tex_size=16) for w in widths]


def test_phased_bytes_tile_pass_writes_every_pixel_with_tensor_maps():
    sc = _scenes([64, 128])
    px = sum(s.width * s.height for s in sc)
    pb = bench.batch_phase_bytes(sc, frags=100.0, tiles=24, dirty=5, phased=True)
    assert pb["clear"] == 0.0
    v = sum(s.mesh.positions.shape[0] for s in sc)
    tex = pb["tile"] - (8.0 * px + 4.0 * 24 + 16.0 * 100 + 48.0 * v)
    assert 0.0 <= tex <= 4.0 * 100 + 1e-9  # min(texture, 4 per covered fragment) over the draws


def test_phased_bytes_clear_kernel_for_widths_without_tensor_maps():
    sc = _scenes([64, 66])  # 66 % 4 != 0: no tensor maps, the clear kernel writes it
    apart = 66 * 32
    px = 64 * 32 + apart
    pb = bench.batch_phase_bytes(sc, frags=0.0, tiles=12, dirty=3, phased=True)
    assert pb["clear"] == 8.0 * apart
    v = sum(s.mesh.positions.shape[0] for s in sc)
    written = 8.0 * (px - apart) + 8.0 * 256 * 3 * apart / px
    assert pb["tile"] == pytest.approx(written + 4.0 * 12 + 48.0 * v)
    # the persistent form writes every pixel in its tile phase
    pp = bench.batch_phase_bytes(sc, frags=0.0, tiles=12, dirty=3, phased=False)
    assert pp["clear"] == 0.0 and pp["tile"] == pytest.approx(8.0 * px + 4.0 * 12 + 48.0 * v)


def test_binned_bytes_are_the_frame_bytes():
    sc = _scenes([64, 128])
    pb = bench.binned_phase_bytes(sc, shaded=50.0)
    v = sum(s.mesh.positions.shape[0] for s in sc)
    f = sum(s.mesh.indices.shape[0] for s in sc)
    px = sum(s.width * s.height for s in sc)
    assert pb["vertex"] == 32.0 * v and pb["face"] == 12.0 * f
    assert 8.0 * px <= pb["tile"] <= 8.0 * px + 4.0 * 50 + 1e-9
    assert pb["clear"] == pb["large"] == 0.0


def test_serve_scalars_flatten_both_modes():
    modes = {m: {"rates": [{"offered_rps": 100.0, "p50_ms": 1.0, "p99_ms": 2.0, "achieved_fps": 99.0},
                           {"offered_rps": 5000.0, "p50_ms": 3.0, "p99_ms": 4.0, "achieved_fps": 4990.0}]}
             for m in ("batched", "per_request")}
    out = bench.serve_scalars(modes)
    assert out["serve_batched_p99_ms_5000rps"] == 4.0 and out["serve_per_req_p50_ms_100rps"] == 1.0
    assert out["serve_batched_fps_100rps"] == 99.0
    assert len(out) == 12
