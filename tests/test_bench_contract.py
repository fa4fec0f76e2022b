"""The bench.py output contract: one JSON line with the keys a reader of the results
relies on, from the reference arm (CPU, here) and from our arm on a reduced batch (GPU)."""
import json
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
BASE_KEYS = {"metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
             "vs_baseline", "dtype", "data", "config", "e2e"}


def run_bench(*args, timeout=600):
    out = subprocess.run([sys.executable, str(ROOT / "bench.py"), *args], cwd=ROOT, capture_output=True, text=True,
                         timeout=timeout, check=True).stdout
    lines = [ln for ln in out.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, out
    return json.loads(lines[0])


def test_reference_arm_line():
    d = run_bench("--impl", "reference", "--steps", "1", "--warmup", "1", "--draws", "64")
    assert BASE_KEYS <= set(d) and d["impl"] == "reference"
    assert d["value"] > 0 and d["metric"] == "frames/s" and d["higher_is_better"] is True
    assert d["cpu_baseline"]["value"] == d["value"] and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0


@pytest.mark.gpu
def test_our_arm_line_on_a_reduced_batch():
    d = run_bench("--draws", "32", "--scale", "0.25", "--steps", "3", "--warmup", "3", "--no-cpu-baseline",
                  timeout=900)
    assert BASE_KEYS <= set(d) and d["value"] > 0
    assert {"roofline", "frame_roofline", "clocks", "gpu_launches", "plain", "batched_vs_plain", "e2e_png",
            "e2e_rgb"} <= set(d)
    r = d["roofline"]
    assert r["bound"] == "hbm" and 0 < r["frac"] < 2 and r["peak"] > 0 and r["achieved"] > 0
    # phased: vertex, face, large, tile per step (a clear kernel too for framebuffers
    # without tensor maps); binned: vertex, face, bin; persistent: one cooperative launch
    assert d["gpu_launches"] in (3 * 5, 3 * 4, 3 * 3, 3 * 1)
    assert d["e2e"]["d2h_bytes_per_step"] > 0 and d["e2e"]["value"] > 0
