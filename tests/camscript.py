"""Seeded camera scripts for the Camera parity tests: sequences of the reference Camera's
operations (rows of 6 floats: kind, a0..a3, flags) and a runner that applies them to the
library's camera (axr_camera_state through axiomr_gb300.api.Camera).

kinds: 0 update(dt); 1 handleInput(mouse a0, a1; flags bit 0 right button, bits 1-4 keys
W S A D); 2 setPosition; 3 setTarget; 4 setFov; 5 setAspectRatio; 6 setViewport."""
from __future__ import annotations

import numpy as np

KEYS = "WSAD"


def script(seed: int, n: int = 60) -> np.ndarray:
    rng = np.random.default_rng(seed)
    ops = []
    mouse = rng.uniform(0, 800, 2)
    for _ in range(n):
        r = rng.random()
        if r < 0.35:
            ops.append([0, rng.choice([0.0, 1 / 60, 1 / 30, 0.1, rng.uniform(0, 0.5)]), 0, 0, 0, 0])
        elif r < 0.75:
            mouse = mouse + rng.normal(0, 25, 2) * (rng.random() < 0.8)
            flags = int(rng.random() < 0.6) | (int(rng.integers(0, 16)) << 1)
            ops.append([1, mouse[0], mouse[1], 0, 0, flags])
        elif r < 0.82:
            ops.append([2, *rng.uniform(-5, 5, 3), 0, 0])
        elif r < 0.89:
            ops.append([3, *rng.uniform(-5, 5, 3), 0, 0])
        elif r < 0.93:
            ops.append([4, rng.uniform(-10, 200), 0, 0, 0, 0])
        elif r < 0.97:
            ops.append([5, rng.uniform(-1, 3), 0, 0, 0, 0])
        else:
            ops.append([6, *rng.integers(0, 100, 2), *rng.integers(1, 2000, 2), 0])
    return np.asarray(ops, np.float32)


def run(cam, ops) -> np.ndarray:
    """Apply the ops to an api.Camera (made with update=False); (n, 51): view, projection,
    viewProjection, position after each op."""
    out = np.zeros((len(ops), 51), np.float32)
    for i, o in enumerate(np.asarray(ops, np.float32)):
        k = int(o[0])
        if k == 0:
            cam.update(o[1])
        elif k == 1:
            f = int(o[5])
            cam.handleInput((o[1], o[2]), bool(f & 1), "".join(c for b, c in enumerate(KEYS) if f & (2 << b)))
        elif k == 2:
            cam.setPosition(o[1:4])
        elif k == 3:
            cam.setTarget(o[1:4])
        elif k == 4:
            cam.setFov(o[1])
        elif k == 5:
            cam.setAspectRatio(o[1])
        elif k == 6:
            cam.setViewport(int(o[1]), int(o[2]), int(o[3]), int(o[4]))
        out[i, 0:16] = cam.view
        out[i, 16:32] = cam.projection
        out[i, 32:48] = cam.view_proj
        out[i, 48:51] = cam.position
    return out


STARTS = [((0.0, 0.0, 3.0), (0.0, 0.0, 0.0), 60.0, 1.0),
          ((1.5, 2.0, -4.0), (0.2, -0.3, 0.5), 75.0, 16.0 / 9.0),
          ((0.0, 5.0, 0.0), (0.0, 0.0, 0.0), 45.0, 4.0 / 3.0),
          ((0.0, 0.0, 0.0), (0.0, 0.0, 1.0), 90.0, 0.5)]
