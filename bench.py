#!/usr/bin/env python3
"""Headline benchmark: frames/s of the AxiomR draw path on one GB300.

A frame is what the reference renderer produces per mesh (src/renderer.cpp:124-126):
clearColor + clearDepth + drawMesh, through the C ABI.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload batch|heightfield|sphere|soup] [--no-autotune]

Default workload `batch`: a step renders the 512 draws of the mixed batch, each into its
own framebuffer, with the batched form (one set of launches over all draws, replayed from
a CUDA graph; launch form and raster parameter autotuned); the plain per-draw path on
the same draws is timed beside it (`plain`, `batched_vs_plain`). The single-draw workloads
(`heightfield`, `sphere`, `soup`) time one frame per step through the per-draw path.

`value` is frames/s with every input resident in HBM; L2 is flushed (a 256 MiB write) before
each timed step and each step is timed with CUDA events on the library's stream. `e2e` is
the same metric with the step's inputs sent from host memory and its results read back
to pinned memory, all inside the timed region (batch: the draw table through
axr_draw_batch up, the 512 rendered images (colour planes) down; single draws: mesh
arrays and texture up, colour and depth down).
`--impl reference` times the CPU restatement of the reference's TiledPipeline (oracle/port,
all host threads) on the same workload instead. With N > 1 (torchrun), every rank renders
its own replica of the workload (the path has no cross-GPU exchange); value is the total.
"""
from __future__ import annotations

import argparse
import ctypes as C
import gc
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

import numpy as np  # noqa: E402

from axiomr_gb300 import workloads as W  # noqa: E402

WORKLOADS = {
    "heightfield": (W.heightfield_scene,
                    "heightfield 1024x1024 vertices (2,093,058 triangles), 2048^2 RGBA8 noise texture, "
                    "Blinn-Phong, camera 30 deg elevation at distance 2.5, 1920x1080"),
    "sphere": (W.sphere_scene, "UV sphere 64x32 (3,968 triangles), 256^2 RGBA8 noise texture, Blinn-Phong, "
                               "camera at distance 3, 512x512"),
    "soup": (W.soup_scene, "200,000 screen-space triangles (edges 0.5-4 px, depths 0.1-100), Gouraud, 3840x2160"),
    "batch": (W.batch_scenes, "512 draws, each a UV sphere with segments log-uniform 8x4..256x128 (48..65,024 "
                              "triangles), resolution uniform from {256^2, 512^2, 1024^2, 1920x1080}, camera on a "
                              "random orbit at distance 2-6, one of 8 1024^2 RGBA8 noise textures, Blinn-Phong"),
}
WORKLOADS["serve"] = (None, "open-loop Poisson arrivals; 90% requests of the small-triangle configuration (200,000 "
                            "triangles, 3840x2160, Gouraud; one of 64 seeded soups), 10% heightfields (2,093,058 "
                            "triangles, 1920x1080, Blinn-Phong, random camera azimuth); 40 GB residency budget")
BATCH_REF_SAMPLE = 16  # draws of the mixed batch the CPU arms render per step (every 32nd)
# FP32 operations of fragment_shader<kBlinnPhong> (axiomr_gb300/csrc/shade.cuh), counted from
# the source: uv barycentric 10, texel scale 6, normal barycentric + normalize 25, world
# position 15, view direction 13, half vector 13, ambient 3, diffuse 9, specular 14,
# combine 9, quantisation 12.
K_BLINN_PHONG = 129
L2_FLUSH_BYTES = 256 << 20


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=("ours", "reference"), default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="batch")
    ap.add_argument("--no-autotune", action="store_true", help="batch: plan with the default tuning table")
    ap.add_argument("--form", choices=("auto", "persistent", "phased", "binned"), default="auto",
                    help="batch: launch form (auto: the autotuner's choice)")
    ap.add_argument("--draw-form", choices=("binned", "keyed"), default="keyed",
                    help="single-draw workloads: form of the per-draw path")
    ap.add_argument("--draws", type=int, default=512, help="batch: number of draws (a smaller batch for profiling)")
    ap.add_argument("--scale", type=float, default=1.0, help="batch: framebuffer size scale (profiling)")
    ap.add_argument("--rates", default="100,500,2000,5000", help="serve: offered loads, requests/s")
    ap.add_argument("--serve-seconds", type=float, default=30.0, help="serve: duration of each offered load")
    ap.add_argument("--budget-gb", type=float, default=40.0, help="serve: device-memory residency budget")
    ap.add_argument("--readback", choices=("colour", "png", "none"), default="colour",
                    help="serve: read each request's colour plane back to host memory, or not")
    ap.add_argument("--serve-mix", choices=("soup", "c4"), default="soup",
                    help="serve: common requests are 3840x2160 soups, or draws of the mixed batch")
    ap.add_argument("--serve-overlap", type=int, choices=(0, 1), default=0,
                    help="serve: 1 = each in-flight batch renders on its own stream (kernels side by side)")
    ap.add_argument("--brief-serve-seconds", type=float, default=3.0,
                    help="batch: seconds per offered load of the short serving sweep in the line (0: none)")
    ap.add_argument("--cpu-budget-s", type=float, default=20.0, help="CPU baseline sample budget")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--profile-range", action="store_true",
                    help="bracket the device-resident timed steps with cudaProfilerStart/Stop (for ncu "
                         "--profile-from-start off: -k <kernel> -c 1 then captures a timed launch)")
    return ap.parse_args()


# ------------------------------------------------------------------ distributed plumbing
class Dist:
    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local_rank = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist

            backend = os.environ.get("AXR_DIST_BACKEND") or ("nccl" if self._cuda() else "gloo")
            if backend == "nccl":
                import torch

                torch.cuda.set_device(self.local_rank)
            dist.init_process_group(backend)
            self.pg = dist

    @staticmethod
    def _cuda():
        try:
            import torch

            return torch.cuda.is_available()
        except Exception:
            return False

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, x: float) -> float:
        if not self.pg:
            return x
        import torch

        dev = f"cuda:{self.local_rank}" if self.pg.get_backend() == "nccl" else "cpu"
        t = torch.tensor([x], dtype=torch.float64, device=dev)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


def aggregate(step_ms: list, dist: Dist):
    """Whole-job frames/s: all ranks' frames over the slowest rank's timed total."""
    total_ms = dist.max(float(sum(step_ms)))
    frames = len(step_ms) * dist.world
    return frames / (total_ms / 1e3), total_ms / len(step_ms)


# ------------------------------------------------------------------ clocks
class ClockSampler:
    """nvidia-smi samples every 200 ms during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    NAMES = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.lines = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-lms", "200", "-i", str(self.device)], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except Exception:
            self.proc = None
        time.sleep(0.3)

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons, power = [], [], set(), []
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
                power.append(float(f[3]))
            except ValueError:
                continue
            for name, v in zip(self.NAMES, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "power_w_max": max(power) if power else None, "samples": len(sm)}


# ------------------------------------------------------------------ helpers
def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            d = json.loads(p.read_text())
            return float(d["hbm_gbs"]), "measured"
        except Exception:
            pass
    return 6800.0, "fallback"


def profiled_traffic(kernel: str, workload: str):
    """DRAM bytes of `kernel` from the committed ncu summary, if any: per launch, or per step
    where a step launches it more than once (the batched form's two launch sets)."""
    f = ROOT / "profiles" / f"{kernel}_{workload}.txt"
    if not f.exists():
        return None
    for line in f.read_text().splitlines():
        if line.startswith("dram_bytes_per_launch:") or line.startswith("dram_bytes_per_step:"):
            try:
                return float(line.split(":", 1)[1].split()[0])
            except ValueError:
                return None
    return None


def pinned_like(lib, arr: np.ndarray, keep: list) -> np.ndarray:
    """Copy `arr` into page-locked host memory from the library's allocator."""
    p = lib.axr_host_alloc(arr.nbytes)
    if not p:
        raise MemoryError("axr_host_alloc failed")
    keep.append(p)
    buf = (C.c_uint8 * arr.nbytes).from_address(p)
    out = np.frombuffer(buf, dtype=arr.dtype).reshape(arr.shape)
    out[...] = arr
    return out


def pinned_bytes(lib, nbytes: int, keep: list) -> np.ndarray:
    """Uninitialised page-locked host bytes from the library's allocator."""
    p = lib.axr_host_alloc(nbytes)
    if not p:
        raise MemoryError("axr_host_alloc failed")
    keep.append(p)
    return np.frombuffer((C.c_uint8 * nbytes).from_address(p), dtype=np.uint8)


def cpu_baseline(scene, steps: int, budget_s: float):
    """The CPU restatement of the reference pipeline (oracle/port) on all host threads."""
    from oracle import Oracle

    port = Oracle("port")
    threads = os.cpu_count() or 1
    vp = port.camera(scene.camera)[2]
    t0 = time.perf_counter()
    port.draw(scene, vp, threads=threads)  # warm-up frame, also sizes the sample
    t1 = time.perf_counter() - t0
    frames = max(1, min(steps, int(budget_s / max(t1, 1e-6))))
    times = []
    for _ in range(frames):
        t = time.perf_counter()
        port.draw(scene, vp, threads=threads)
        times.append(time.perf_counter() - t)
    value = len(times) / sum(times)
    return {"value": value, "unit": "frames/s", "cores": threads, "kind": "port",
            "sample": f"{len(times)} full frames of the workload (clear excluded), median "
                      f"{statistics.median(times) * 1e3:.1f} ms/frame, host {os.uname().machine}"}


# ------------------------------------------------------------------ GPU arm
def run_ours(args, dist: Dist):
    import torch

    from axiomr_gb300 import api

    make, desc = WORKLOADS[args.workload]
    scene = make()
    dev = dist.local_rank
    torch.cuda.set_device(dev)
    ctx = api.Context(dev)
    ctx.draw_form = api.DRAW_KEYED if args.draw_form == "keyed" else api.DRAW_BINNED
    lib = ctx.lib
    fb = api.Framebuffer(ctx, scene.width, scene.height)
    textures = {}
    m = scene.mesh
    shader_kind = scene.shader.kind
    need_tbn = shader_kind in (W.SHADER_PHONG, W.SHADER_PBR)
    mats = []
    images = {}

    def tex(img):
        if img is None:
            return None
        if id(img) not in textures:
            textures[id(img)] = api.Texture(ctx, img)
            images[id(img)] = img
        return textures[id(img)]

    for mat in m.materials:
        mats.append(api.Material(tex(mat.diffuse), tex(mat.bump), tex(mat.metallic), tex(mat.roughness), tex(mat.ao),
                                 mat.specular_exponent))
    mesh = api.Mesh(ctx, m.positions, m.uvs, m.normals, m.indices, m.groups, mats,
                    m.tangents if need_tbn else None, m.bitangents if need_tbn else None)
    cam = api.Camera.from_workload(scene.camera)
    pipe = api.TiledPipeline(ctx, cam, fb)
    sh = scene.shader
    pipe.setShader(api.Shader(sh.kind, tuple(sh.light_direction), tuple(sh.light_color)))
    model = np.asarray(scene.model, np.float32)
    b, g, r, a = scene.clear_bgra
    stream = torch.cuda.ExternalStream(ctx.stream, device=f"cuda:{dev}")
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=f"cuda:{dev}")

    def frame():
        fb.clearColor(r, g, b, a)
        fb.clearDepth()
        pipe.drawMesh(model, mesh)

    for _ in range(max(3, args.warmup)):
        frame()
    ctx.sync()

    # untimed statistics pass: rasterised fragments and surviving triangles per frame
    ctx.stats(True)
    ctx.stats()
    frame()
    st = ctx.stats()
    ctx.stats(False)

    # ---- timed: inputs resident in HBM
    ctx.profile(True)
    launches0 = ctx.profile()["kernel_launches"]
    sampler = ClockSampler(dev)
    dist.barrier()
    torch.cuda.synchronize()
    ctx.sync()
    sampler.start()
    evs = []
    if args.profile_range:
        torch.cuda.profiler.start()
    for _ in range(args.steps):
        with torch.cuda.stream(stream):
            flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        frame()
        e1.record(stream)
        evs.append((e0, e1))
    ctx.sync()
    torch.cuda.synchronize()
    if args.profile_range:
        torch.cuda.profiler.stop()
    dist.barrier()
    sampler.stop()
    step_ms = [e0.elapsed_time(e1) for e0, e1 in evs]
    prof = ctx.profile()
    ctx.profile(False)
    launches = prof["kernel_launches"] - launches0
    value, ms_per_step = aggregate(step_ms, dist)
    if args.profile_range:  # a profiling run: the captured frames are all it is for
        return {"profile_range": True, "workload": args.workload, "ms_per_step": round(ms_per_step, 4)}, scene

    # ---- timed end to end: uploads from pinned host memory and read-back in the region
    keep = []
    h_pos = pinned_like(lib, m.positions, keep)
    h_uv = pinned_like(lib, m.uvs, keep)
    h_nrm = pinned_like(lib, m.normals, keep)
    h_idx = pinned_like(lib, m.indices, keep)
    h_tan = pinned_like(lib, m.tangents, keep) if need_tbn else None
    h_bit = pinned_like(lib, m.bitangents, keep) if need_tbn else None
    tex_list = [textures[k] for k in images]
    h_tex = [pinned_like(lib, np.ascontiguousarray(images[k]), keep) for k in images]
    h_bgra = pinned_like(lib, np.zeros((scene.height, scene.width, 4), np.uint8), keep)
    h_depth = pinned_like(lib, np.zeros((scene.height, scene.width), np.float32), keep)
    h2d = sum(x.nbytes for x in (h_pos, h_uv, h_nrm, h_idx) + tuple(h for h in (h_tan, h_bit) if h is not None))
    h2d += sum(x.nbytes for x in h_tex)
    d2h = h_bgra.nbytes + h_depth.nbytes

    def e2e_frame():
        mesh.update(h_pos, h_uv, h_nrm, h_idx, h_tan, h_bit)
        for t, img in zip(tex_list, h_tex):
            t.update(img)
        frame()
        C_ok = lib.axr_framebuffer_read_async(ctx.handle, fb.handle, h_bgra.ctypes.data, h_depth.ctypes.data)
        if C_ok != 0:
            raise RuntimeError("axr_framebuffer_read_async failed")

    for _ in range(max(3, args.warmup)):
        e2e_frame()
    ctx.sync()
    dist.barrier()
    torch.cuda.synchronize()
    evs = []
    for _ in range(args.steps):
        with torch.cuda.stream(stream):
            flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        e2e_frame()
        e1.record(stream)
        evs.append((e0, e1))
    ctx.sync()
    torch.cuda.synchronize()
    dist.barrier()
    e2e_ms = [e0.elapsed_time(e1) for e0, e1 in evs]
    e2e_value, _ = aggregate(e2e_ms, dist)
    for p in keep:
        lib.axr_host_free(p)

    # ---- roofline of the dominant kernel
    n = max(1, prof["draws"])
    stages = ("vertex", "geometry", "large", "scan", "shade", "clipped")
    stage_us = {k: prof[k + "_ms"] / n * 1e3 for k in stages}
    V, F = m.num_vertices, m.num_faces
    P = scene.width * scene.height
    frags = st["fragments"]
    scanned_px = min(P, st["tiles"] * 256)
    vattr = {W.SHADER_PHONG: 64, W.SHADER_PBR: 64, W.SHADER_BLINN_PHONG: 32}.get(shader_kind, 16)
    vin = 40 + (24 if need_tbn else 0)  # position, normal, uv (+ tangent, bitangent) read per vertex
    algo_bytes = {
        # vertex attributes read once, screen cache (16 B) + shader outputs written once
        "vertex": float(V) * (vin + 16 + vattr),
        # indices read once, cached screen positions read once per vertex, one 8-byte
        # depth-key write per covered fragment
        "geometry": 12.0 * F + 16.0 * V + 8.0 * frags,
        "large": 8.0 * frags,
        # keys of the dirty tiles read, one 8-byte work entry per covered pixel written
        "scan": 8.0 * scanned_px + 8.0 * frags,
        # per covered pixel: work entry, indices, depth read, colour + depth write; the
        # vertex cache read once
        "shade": frags * (8.0 + 12.0 + 4.0 + 8.0) + float(V) * (16 + vattr),
        "clipped": 0.0,
    }
    kernel_names = {k: k + "_kernel" for k in stages}
    kernel_names["clipped"] = "resolve_clipped_kernel"
    if args.draw_form == "binned":
        # three kernels: vertices, faces (setup and binning; the profile's geometry stage) and
        # bins (raster, shading and tile write-out; its shading stage). Algorithmic bytes: the
        # vertex attributes, the indices, and one colour + depth write per pixel plus
        # min(texture, 4 per shaded fragment), each where it moves
        tex_bytes = sum(int(t.nbytes) for t in images.values())
        algo_bytes = {"vertex": float(V) * vin, "geometry": 12.0 * F, "large": 0.0, "scan": 0.0,
                      "shade": 8.0 * P + min(tex_bytes, 4.0 * st["shaded"]), "clipped": 0.0}
        kernel_names = {"vertex": "solo_vertex_kernel", "geometry": "solo_face_kernel", "large": "-", "scan": "-",
                        "shade": "solo_bin_kernel", "clipped": "-"}
    dom = max(stage_us, key=stage_us.get)
    hbm_peak, peak_kind = measured_peaks()
    achieved = algo_bytes[dom] / (stage_us[dom] * 1e-6) / 1e9
    traffic = profiled_traffic(kernel_names[dom], args.workload)
    roofline = {"bound": "hbm", "kernel": kernel_names[dom], "achieved": round(achieved, 1), "peak": hbm_peak,
                "peak_source": peak_kind, "unit": "GB/s", "frac": round(achieved / hbm_peak, 4),
                "traffic": traffic, "algorithmic_bytes": algo_bytes[dom], "launch_us": round(stage_us[dom], 2),
                "stage_us": {k: round(v, 2) for k, v in stage_us.items()}}

    out = {
        "metric": "frames/s", "value": round(value, 2), "unit": "frames/s", "n_gpus": dist.world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_per_step, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded generators in axiomr_gb300/workloads.py)",
        "config": {"workload": f"{args.workload}: {desc}",
                   "form": f"plain (one drawMesh per frame, {args.draw_form} form)",
                   "l2": "flushed before every timed step (256 MiB write, outside the events)",
                   "parallelism": f"replicas x{dist.world}" if dist.world > 1 else "single GPU"},
        "gfrag_per_s": round(frags * value / 1e9, 3),
        "mtri_per_s": round(F * value / 1e6, 2),
        "fragments_per_frame": int(frags), "triangles_per_frame": int(st["triangles"]),
        "e2e": {"value": round(e2e_value, 2), "unit": "frames/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h)},
        "gpu_launches": int(launches),
        "roofline": roofline,
        "clocks": sampler.summary(),
    }
    ctx.close()
    return out, scene


def timed_steps(stream, flush, steps: int, body, profile_range: bool = False):
    """K steps of `body`, each bracketed by CUDA events on the library stream after an L2
    flush (outside the events); returns per-step milliseconds. With profile_range the steps
    run between cudaProfilerStart and cudaProfilerStop."""
    import torch

    evs = []
    if profile_range:
        torch.cuda.profiler.start()
    for _ in range(steps):
        with torch.cuda.stream(stream):
            flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        body()
        e1.record(stream)
        evs.append((e0, e1))
    torch.cuda.synchronize()
    if profile_range:
        torch.cuda.profiler.stop()
    return [a.elapsed_time(b) for a, b in evs]


def batch_config(args, dist: "Dist", frames: int) -> dict:
    """The mixed-batch workload as both arms describe it (identical dictionaries, so that
    the two lines name the same configuration); how each arm renders it is reported
    outside `config`."""
    desc = WORKLOADS["batch"][1]
    if args.draws != 512 or args.scale != 1.0:
        desc += f" [reduced: first {args.draws} draws, framebuffers scaled by {args.scale}]"
    return {"workload": f"batch: {desc}", "frames_per_step": frames, "draws": args.draws, "resolution_scale": args.scale,
            "l2": "flushed before every timed step (256 MiB write, outside the events); inputs larger than L2",
            "parallelism": f"replicas x{dist.world}" if dist.world > 1 else "single GPU"}


def batch_algo_bytes(scenes, frags: float) -> float:
    """Algorithmic bytes of one mixed-batch step: per draw the vertex attributes read
    (position 12 + normal 12 + uv 8), the indices (12 per face), one colour + one depth
    write per pixel, and min(texture bytes, 4 per covered fragment) summed over draws
    (covered fragments split by faces)."""
    total_faces = sum(int(sc.mesh.indices.shape[0]) for sc in scenes)
    b = 0.0
    for sc in scenes:
        V, F = sc.mesh.positions.shape[0], sc.mesh.indices.shape[0]
        tex = sum(int(t.nbytes) for m in sc.mesh.materials for t in (m.diffuse,) if t is not None)
        b += 32.0 * V + 12.0 * F + 8.0 * sc.width * sc.height + min(tex, 4.0 * frags * F / max(1, total_faces))
    return b


def binned_phase_bytes(scenes, shaded: float) -> dict:
    """Algorithmic bytes of each phase of one step in the binned form, the frame's bytes
    split by the phase that moves them: the vertex attributes read (32 per vertex:
    position, normal, uv) by the vertex phase, the indices (12 per face) by the face phase,
    and one colour + one depth write per pixel (8) plus min(texture bytes, 4 per shaded
    fragment) by the bin pass. Their sum is the frame roofline's bytes; the intermediate
    data of the design (vertex cache, raster records, bin entries) is not counted, so the
    measured traffic against these figures shows its cost."""
    total_faces = sum(int(sc.mesh.indices.shape[0]) for sc in scenes)
    v = f = px = tex = 0.0
    for sc in scenes:
        V, F = sc.mesh.positions.shape[0], sc.mesh.indices.shape[0]
        t = sum(int(m.diffuse.nbytes) for m in sc.mesh.materials if m.diffuse is not None)
        v += V
        f += F
        px += sc.width * sc.height
        tex += min(t, 4.0 * shaded * F / max(1, total_faces))
    return {"clear": 0.0, "vertex": 32.0 * v, "face": 12.0 * f, "large": 0.0, "tile": 8.0 * px + tex}


def batch_phase_bytes(scenes, frags: float, tiles: int, dirty: int, phased: bool) -> dict:
    """Algorithmic bytes of each phase of one batched step (Blinn-Phong: 48-byte vertex
    cache entries): vertices read (32) + cache written (48) per vertex; indices (12 per
    face) + cache gathers (16 per vertex) + one key per covered fragment (8) for the face
    and large phases together; the tile pass reads the flags (4 per tile), reads and resets
    the key of every covered pixel (16), reads the vertex cache (48 per vertex) and
    min(texture, 4 per covered fragment), and writes colour + depth (8 per pixel) of every
    pixel, except in the phased form for framebuffers without tensor maps (width not a
    multiple of 4): a clear kernel writes those (its own 8 per pixel) and the tile pass
    only their dirty tiles."""
    total_faces = sum(int(sc.mesh.indices.shape[0]) for sc in scenes)
    v = f = px = tex = apart = 0.0
    for sc in scenes:
        V, F = sc.mesh.positions.shape[0], sc.mesh.indices.shape[0]
        t = sum(int(m.diffuse.nbytes) for m in sc.mesh.materials if m.diffuse is not None)
        v += V
        f += F
        px += sc.width * sc.height
        if phased and sc.width % 4 != 0:
            apart += sc.width * sc.height
        tex += min(t, 4.0 * frags * F / max(1, total_faces))
    written = 8.0 * (px - apart) + (8.0 * 256 * dirty * apart / px if px else 0.0)
    return {"clear": 8.0 * apart, "vertex": 80.0 * v,
            "face": 12.0 * f + 16.0 * v + 8.0 * frags, "large": 8.0 * frags,
            "tile": written + 4.0 * tiles + 16.0 * frags + 48.0 * v + tex}


def run_batch_png(ctx, lib, stream, flush, sets, tables, args, dist, keep) -> dict:
    """End to end with PNG output, pipelined: two framebuffer sets; step k renders set k%2
    (axr_draw_batch), enqueues its PNG encode (axr_png_batch_encode) and then copies the
    files of step k-1 to pinned memory (axr_png_batch_read) while the GPU works on step k.
    Timed over K steps plus the last read. Also the encode alone on the device (CUDA
    events), against the HBM peak with its algorithmic bytes: each colour plane read once
    (4 per pixel) and each file written."""
    import torch

    from axiomr_gb300 import api

    draws = sets[0]
    n = len(draws)
    fb_lists = [(C.c_void_p * n)(*[d.framebuffer.handle.value for d in st]) for st in sets]
    caps = [api.png_bound(d.framebuffer.width, d.framebuffer.height, 3) for d in draws]
    host = [[pinned_bytes(lib, c, keep) for c in caps] for _ in sets]
    ptrs = [(C.c_void_p * n)(*[h.ctypes.data for h in hs]) for hs in host]
    capa = (C.c_uint64 * n)(*caps)
    pngs = [api.PngBatch(ctx), api.PngBatch(ctx)]

    def run(steps):
        for k in range(steps):
            cur = k % 2
            api.draw_batch(ctx, tables[cur])
            pngs[cur].encode(fb_lists[cur], 3)
            if k:
                pngs[1 - cur].read_into(ptrs[1 - cur], capa)
        last = (steps - 1) % 2
        pngs[last].read_into(ptrs[last], capa)

    run(4)
    torch.cuda.synchronize()
    steps = max(3, args.steps // 2)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    dist.barrier()
    e0.record(stream)
    run(steps)
    e1.record(stream)
    torch.cuda.synchronize()
    total_ms = dist.max(float(e0.elapsed_time(e1)))
    value = n * steps * dist.world / (total_ms / 1e3)
    sizes = pngs[0].sizes()
    file_bytes = int(sum(sizes))
    pixels = sum(d.framebuffer.width * d.framebuffer.height for d in draws)
    # the encode alone, into device buffers
    bufs = [torch.empty((c + 255) // 256 * 256, dtype=torch.uint8, device=f"cuda:{dist.local_rank}") for c in caps]
    dsz = torch.zeros(n, dtype=torch.int64, device=f"cuda:{dist.local_rank}")
    outs = (C.c_void_p * n)(*[b.data_ptr() for b in bufs])
    fb_arr = (C.c_void_p * n)(*[d.framebuffer.handle.value for d in draws])
    torch.cuda.synchronize()

    def encode():
        rc = lib.axr_framebuffers_encode_png(ctx.handle, n, fb_arr, 3, outs, capa, C.c_void_p(dsz.data_ptr()))
        if rc != 0:
            raise RuntimeError("axr_framebuffers_encode_png failed")

    for _ in range(3):
        encode()
    enc_ms = timed_steps(stream, flush, max(3, args.steps // 2), encode)
    enc = sum(enc_ms) / len(enc_ms)
    hbm_peak, peak_kind = measured_peaks()
    algo = 4.0 * pixels + file_bytes
    del bufs
    for pb in pngs:
        pb.close()
    return {"value": round(value, 2), "unit": "frames/s", "h2d_bytes_per_step": int(n * C.sizeof(api.DrawDesc)),
            "d2h_bytes_per_step": file_bytes + 8 * n,
            "path": "per step: axr_draw_batch + axr_png_batch_encode of the 512 frames (RGB PNG files, encoded on "
                    "the GPU, lossless), while the previous step's files are copied to pinned memory "
                    "(axr_png_batch_read); two framebuffer sets, inputs larger than L2",
            "steps": steps, "png_bytes_per_step": file_bytes, "rgb_bytes_per_step": 3 * pixels,
            "encode_us": round(enc * 1e3, 2), "encode_launches": 4,
            "encode_roofline": {"bound": "hbm", "achieved": round(algo / (enc * 1e-3) / 1e9, 1), "peak": hbm_peak,
                                "peak_source": peak_kind, "unit": "GB/s",
                                "frac": round(algo / (enc * 1e-3) / 1e9 / hbm_peak, 4), "algorithmic_bytes": algo,
                                "definition": "4 bytes per pixel read + the file bytes written"}}


def run_batch(args, dist: Dist):
    """The mixed batch: 512 draws into 512 framebuffers per step, batched form (one
    persistent launch, replayed from a CUDA graph) against the plain per-draw path (clear,
    clear, drawMesh per draw, also replayed from a CUDA graph)."""
    import torch

    from axiomr_gb300 import api

    scenes = W.batch_scenes(count=args.draws, resolution_scale=args.scale)
    dev = dist.local_rank
    torch.cuda.set_device(dev)
    ctx = api.Context(dev)
    lib = ctx.lib
    textures, meshes = {}, {}
    draws = api.batch_draws(ctx, scenes, textures, meshes)
    stream = torch.cuda.ExternalStream(ctx.stream, device=f"cuda:{dev}")
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=f"cuda:{dev}")
    n = len(draws)

    # ---- the step with the default tuning table and launch form, for comparison
    form_names = {api.BATCH_PERSISTENT: "persistent", api.BATCH_PHASED: "phased", api.BATCH_BINNED: "binned"}
    untuned = None
    if not args.no_autotune and not args.profile_range:
        b0 = api.Batch(ctx, draws)
        g0 = api.Graph(ctx).begin()
        b0.launch()
        g0.end()
        for _ in range(3):
            g0.launch()
        ctx.sync()
        ms0 = timed_steps(stream, flush, max(3, args.steps // 2), g0.launch)
        untuned = {"ms_per_step": round(sum(ms0) / len(ms0), 4), "form": form_names[b0.info()["form"]],
                   "tuning_small_max_pixels": ctx.tuning(), "tuning_bins": ctx.bin_tuning()}
        g0.close()
        b0.close()

    # ---- autotune the per-class raster parameters and the launch form on this batch, then plan it
    tuning = ctx.tuning() if args.no_autotune else api.autotune(ctx, draws, repeats=2)
    if args.form != "auto":
        ctx.batch_form = {"persistent": api.BATCH_PERSISTENT, "phased": api.BATCH_PHASED,
                          "binned": api.BATCH_BINNED}[args.form]
    batch = api.Batch(ctx, draws)
    info = batch.info()
    k0 = ctx.profile()["kernel_launches"]
    graph = api.Graph(ctx).begin()
    batch.launch()
    graph.end()
    kernels_per_step = ctx.profile()["kernel_launches"] - k0  # the kernels one replay runs

    # ---- plain per-draw path, recorded once into a graph as well
    ctx.reserve(max(int(sc.mesh.indices.shape[0]) for sc in scenes))
    pipe = api.TiledPipeline(ctx)
    plain_graph = api.Graph(ctx).begin()
    for d in draws:
        d.framebuffer.clearColor(*d.clear_color)
        d.framebuffer.clearDepth(d.clear_depth)
        pipe.setCamera(d.camera)
        pipe.setFramebuffer(d.framebuffer)
        pipe.setShader(d.shader)
        pipe.drawMesh(d.model, d.mesh)
    plain_graph.end()
    launches0 = ctx.profile()["kernel_launches"]
    for d in draws[:1]:
        pipe.setCamera(d.camera)
        pipe.setFramebuffer(d.framebuffer)
        pipe.setShader(d.shader)
        d.framebuffer.clearColor(*d.clear_color)
        d.framebuffer.clearDepth(d.clear_depth)
        pipe.drawMesh(d.model, d.mesh)
    plain_launches_per_draw = ctx.profile()["kernel_launches"] - launches0  # clears included
    ctx.sync()

    # statistics of one batched step
    ctx.stats(True)
    ctx.stats()
    batch.launch()
    st = ctx.stats()
    ctx.stats(False)

    for _ in range(max(3, args.warmup)):
        graph.launch()
        plain_graph.launch()
    ctx.sync()

    sampler = ClockSampler(dev)
    dist.barrier()
    torch.cuda.synchronize()
    sampler.start()
    step_ms = timed_steps(stream, flush, args.steps, graph.launch, args.profile_range)
    dist.barrier()
    sampler.stop()
    if args.profile_range:  # a profiling run: the captured steps are all it is for
        return {"profile_range": True, "form": info["form"], "ms_per_step": round(sum(step_ms) / len(step_ms), 4),
                "config": batch_config(args, dist, n)}, scenes
    plain_ms = timed_steps(stream, flush, args.steps, plain_graph.launch)
    # the plain path as a host loop of per-draw calls (no graph), for reference
    eager_ms = timed_steps(stream, flush, max(3, args.steps // 4), lambda: [
        (d.framebuffer.clearColor(*d.clear_color), d.framebuffer.clearDepth(d.clear_depth), pipe.setCamera(d.camera),
         pipe.setFramebuffer(d.framebuffer), pipe.setShader(d.shader), pipe.drawMesh(d.model, d.mesh))
        for d in draws])
    ctx.sync()
    total_ms = dist.max(float(sum(step_ms)))
    value = n * len(step_ms) * dist.world / (total_ms / 1e3)
    plain_value = n * len(plain_ms) / (sum(plain_ms) / 1e3)
    eager_value = n * len(eager_ms) / (sum(eager_ms) / 1e3)

    # ---- end to end. The step's result is the 512 rendered images: per step the draw table
    # goes up from the host (the one-shot batch entry point) and the colour planes come back
    # to pinned host memory (the depth planes stay on the device, as the reference's
    # framebuffer keeps its depth). Serial: draw, read back, next step. Pipelined: two
    # framebuffer sets; step k renders set k%2 and starts its read-back on the read-back's
    # own copy streams (axr_readback_start), then waits for step k-1's (axr_readback_wait),
    # so the copies of one step overlap the rendering of the next.
    keep = []
    sets = [draws, api.batch_draws(ctx, scenes, textures, meshes)]
    tables = [api.draw_table(st) for st in sets]  # the host program's draw tables, uploaded every step
    fb_arrs = [(C.c_void_p * n)(*[d.framebuffer.handle.value for d in st]) for st in sets]
    outs = [[pinned_bytes(lib, d.framebuffer.width * d.framebuffer.height * 4, keep) for d in draws] for _ in sets]
    bgra_arrs = [(C.c_void_p * n)(*[hb.ctypes.data for hb in o]) for o in outs]
    d2h = sum(a.nbytes for a in outs[0])
    h2d = n * C.sizeof(api.DrawDesc)
    fb_arr = fb_arrs[0]

    def e2e_step():
        api.draw_batch(ctx, tables[0])
        rc = lib.axr_framebuffers_read_async(ctx.handle, n, fb_arrs[0], bgra_arrs[0], None)
        if rc != 0:
            raise RuntimeError("axr_framebuffers_read_async failed")

    for _ in range(2):
        e2e_step()
    ctx.sync()
    serial_ms = timed_steps(stream, flush, max(5, args.steps // 2), e2e_step)
    serial_value = n * dist.world / (dist.max(float(np.median(serial_ms))) / 1e3)  # median step

    rbs = []
    for _ in sets:
        h = C.c_void_p()
        api.check(lib.axr_readback_create(ctx.handle, C.byref(h)), ctx.handle)
        rbs.append(h)

    # the packed read-back: all planes gathered on the device, one block per step into one
    # pinned buffer per set (BGRA as stored, or RGB top row first as the window shows them)
    pixels = sum(d.framebuffer.width * d.framebuffer.height for d in draws)
    packed = {fmt: [pinned_bytes(lib, pixels * bpp, keep) for _ in sets] for fmt, bpp in ((0, 4), (1, 3))}

    def start_planes(cur):
        api.check(lib.axr_readback_start(ctx.handle, rbs[cur], n, fb_arrs[cur], bgra_arrs[cur], None), ctx.handle)

    def start_packed(fmt):
        def start(cur):
            buf = packed[fmt][cur]
            api.check(lib.axr_readback_start_packed(ctx.handle, rbs[cur], n, fb_arrs[cur], fmt, buf.ctypes.data,
                                                    buf.nbytes), ctx.handle)
        return start

    def pipelined(steps, start):
        for k in range(steps):
            cur = k % 2
            api.draw_batch(ctx, tables[cur])
            start(cur)
            if k:
                api.check(lib.axr_readback_wait(ctx.handle, rbs[1 - cur]), ctx.handle)
        api.check(lib.axr_readback_wait(ctx.handle, rbs[(steps - 1) % 2]), ctx.handle)

    e2e_steps = max(3, args.steps // 2)

    # The host link is shared with the machine's other GPUs: a neighbour's copies can halve
    # the device-to-host rate for a while. Each figure is therefore the median of five timed
    # windows of e2e_steps steps each, every window's value kept in the line.
    e2e_windows = 5

    def timed_pipeline(start):
        pipelined(4, start)
        torch.cuda.synchronize()
        vals = []
        for _ in range(e2e_windows):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            dist.barrier()
            e0.record(stream)
            pipelined(e2e_steps, start)
            e1.record(stream)
            torch.cuda.synchronize()
            vals.append(n * e2e_steps * dist.world / (dist.max(float(e0.elapsed_time(e1))) / 1e3))
        return float(np.median(vals)), [round(v, 1) for v in vals]

    l0 = ctx.profile()["kernel_launches"]
    e2e_value, e2e_wins = timed_pipeline(start_packed(0))
    e2e_launches = (ctx.profile()["kernel_launches"] - l0) / (e2e_windows * e2e_steps + 4)
    planes_value, planes_wins = timed_pipeline(start_planes)
    rgb_value, rgb_wins = timed_pipeline(start_packed(1))
    for h in rbs:
        lib.axr_readback_destroy(ctx.handle, h)

    # ---- the same, with the frames delivered as PNG files encoded on the GPU (RGB, top row
    # first: the picture the reference's window shows); only the files cross the link
    png = run_batch_png(ctx, lib, stream, flush, sets, tables, args, dist, keep)
    for p in keep:
        lib.axr_host_free(p)

    # per-phase device time of one batch (eager launches with profiling on)
    ctx.profile(True)
    ctx.profile()
    n_prof = 3
    for _ in range(n_prof):
        batch.launch()
    pr = ctx.profile()
    ctx.profile(False)
    # per step: the sum over the step's launches of each phase (a split batch launches every
    # phase once per launch set; with timing on the sets run in turn)
    phase_ms = {k: pr[f"batch_{k}_ms"] / n_prof for k in ("clear", "vertex", "face", "large", "tile")}
    launches_per_step = max(1, pr["batch_launches"] // n_prof)

    fp32_tflops = ctx.fp32_peak_tflops()
    hbm_peak, peak_kind = measured_peaks()
    ms = total_ms / len(step_ms)
    frags = float(st["fragments"])
    algo = batch_algo_bytes(scenes, frags)
    # fragment ALU work (the frame roofline's ALU side): FP32 operations of the Blinn-Phong
    # fragment functor counted from its source (K_BLINN_PHONG) per shaded fragment, plus
    # three edge evaluations and three compares (9) per tested pixel
    alu_flop = K_BLINN_PHONG * float(st["shaded"]) + 9.0 * float(st["tested"])
    alu_tflops = alu_flop / (ms * 1e-3) / 1e12
    achieved = algo / (ms * 1e-3) / 1e9
    faces = info["faces"]
    pb = binned_phase_bytes(scenes, float(st["shaded"])) if info["form"] == 2 else \
        batch_phase_bytes(scenes, frags, int(info["tiles"]), int(st["tiles"]), info["form"] == 1)
    dom = max(phase_ms, key=phase_ms.get)
    kernel_of = {"clear": "-", "vertex": "batch_bin_vertex_kernel", "face": "batch_bin_face_kernel", "large": "-",
                 "tile": "batch_bin_kernel"} if info["form"] == 2 else \
        {"clear": "batch_clear_kernel", "vertex": "batch_vertex_kernel", "face": "batch_face_kernel",
                 "large": "batch_large_kernel", "tile": "batch_tile_kernel"} if info["form"] == 1 else \
        {k: "batch_kernel" for k in phase_ms}
    dom_achieved = pb[dom] / (phase_ms[dom] * 1e-3) / 1e9 if phase_ms[dom] > 0 else 0.0
    # the same pass on the frame's own bytes only (colour + depth of every pixel it writes
    # and the texels), without the design's intermediate data (keys, flags, vertex cache)
    frame_only = binned_phase_bytes(scenes, float(st["shaded"]))["tile"] if dom == "tile" else pb[dom]
    frame_only_achieved = frame_only / (phase_ms[dom] * 1e-3) / 1e9 if phase_ms[dom] > 0 else 0.0
    out = {
        "metric": "frames/s", "value": round(value, 2), "unit": "frames/s", "n_gpus": dist.world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded generators in axiomr_gb300/workloads.py)",
        "config": batch_config(args, dist, n),
        "form_desc": ("batched, binned: three launches over the work units of all draws (vertices; faces, "
                      "set up and binned into bins of 8 tiles; one CTA per bin rasterising it in shared memory, "
                      "shading the winners and writing colour and depth once with TMA stores, clears fused)"
                      + (", as two launch sets of alternating draws on two streams" if info["launches"] > 1 else "")
                      if info["form"] == 2 else
                      "batched, phased: four phase launches (the tile pass also clearing the key-less tiles "
                      "with TMA stores) over the work units of "
                      "all draws, as two launch sets of alternating draws on two streams"
                      if info["form"] == 1 and info["launches"] > 1 else
                      "batched, phased: four phase launches per step (the tile pass also clearing the "
                      "key-less tiles with TMA stores) over the work "
                      "units of all draws" if info["form"] == 1 else
                      "batched, persistent: one cooperative launch per step (clears fused into the tile pass)")
        + ", replayed from a CUDA graph",
        "tuning_small_max_pixels": tuning,
        "tuning_bins": ctx.bin_tuning(),
        "untuned": untuned,
        "tuned_vs_untuned": round(untuned["ms_per_step"] / ms, 3) if untuned else None,
        "gfrag_per_s": round(frags * value / n / 1e9, 3),
        "mtri_per_s": round(faces * value / n / 1e6, 2),
        "fragments_per_step": int(frags), "shaded_per_step": int(st["shaded"]), "tested_per_step": int(st["tested"]),
        "triangles_per_step": int(st["triangles"]), "faces_per_step": int(faces),
        "pixels_per_step": int(info["pixels"]),
        "plain": {"value": round(plain_value, 2), "unit": "frames/s", "ms_per_step": round(sum(plain_ms) / len(plain_ms), 4),
                  "form": "per draw: clearColor, clearDepth, drawMesh (9 launches), replayed from a CUDA graph",
                  "launches_per_draw": int(plain_launches_per_draw)},
        "plain_eager": {"value": round(eager_value, 2), "unit": "frames/s",
                        "form": "the same per-draw calls issued from the Python host loop"},
        "batched_vs_plain": round(value / plain_value, 3),
        "e2e": {"value": round(e2e_value, 2), "unit": "frames/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h),
                # the device-resident comparison the batched form is built for, kept as plain
                # numbers beside the end-to-end figure
                "plain_frames_per_s": round(plain_value, 2), "batched_frames_per_s": round(value, 2),
                "batched_vs_plain": round(value / plain_value, 3),
                "path": "per step axr_draw_batch (draw table from the host) + read-back of all 512 rendered "
                        "images (BGRA8 colour planes, as stored) into one pinned buffer: gathered on the device "
                        "and copied as one block (axr_readback_start_packed / axr_readback_wait), pipelined over "
                        "two framebuffer sets so that step k's copies overlap step k+1's rendering; meshes and "
                        "textures resident; inputs larger than L2",
                "steps": e2e_steps, "windows": e2e_wins,
                "statistic": f"median of {e2e_windows} timed windows of {e2e_steps} steps",
                "d2h_gb_per_s": round(d2h * e2e_value / n / 1e9, 1), "gpu_launches_per_step": e2e_launches,
                "per_plane_copies": {"value": round(planes_value, 2), "unit": "frames/s", "windows": planes_wins,
                                     "path": "the same with one copy per colour plane (axr_readback_start)"},
                "serial": {"value": round(serial_value, 2), "unit": "frames/s",
                           "path": "the same without overlap: draw, read back (axr_framebuffers_read_async), "
                                   "next step; L2 flushed before each step; median step"}},
        "e2e_rgb": {"value": round(rgb_value, 2), "unit": "frames/s", "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(3 * pixels), "windows": rgb_wins,
                    "path": "the e2e pipeline with the frames as RGB8, top row first (the picture the reference's "
                            "window shows), packed on the device: 3 bytes per pixel cross the link"},
        "e2e_png": png,
        "gpu_launches": int(kernels_per_step) * len(step_ms),
        "roofline": {"bound": "hbm", "kernel": kernel_of[dom], "phase": dom, "achieved": round(dom_achieved, 1),
                     "peak": hbm_peak, "peak_source": peak_kind, "unit": "GB/s",
                     "frac": round(dom_achieved / hbm_peak, 4), "traffic": profiled_traffic(kernel_of[dom], "batch"),
                     "algorithmic_bytes": pb[dom], "kernel_us_per_step": round(phase_ms[dom] * 1e3, 2),
                     "frame_bytes_only": frame_only, "frac_frame_bytes_only": round(frame_only_achieved / hbm_peak, 4),
                     "launches_per_step": launches_per_step,
                     "per": "step: algorithmic bytes, traffic and kernel time summed over the step's launches "
                            "of the kernel (one per launch set)",
                     "phase_us": {k: round(v * 1e3, 2) for k, v in phase_ms.items()}},
        "frame_roofline": {"bound": "hbm" if achieved / hbm_peak >= alu_tflops / fp32_tflops else "alu",
                           "hbm": {"achieved": round(achieved, 1), "peak": hbm_peak, "unit": "GB/s",
                                   "frac": round(achieved / hbm_peak, 4), "algorithmic_bytes": algo,
                                   "definition": "per draw V*32 + F*12 + W*H*8 + min(texture, 4 per covered "
                                                 "fragment), over the whole step"},
                           "alu": {"achieved": round(alu_tflops, 3), "peak": round(fp32_tflops, 2), "unit": "TFLOP/s",
                                   "frac": round(alu_tflops / fp32_tflops, 4), "flop": alu_flop,
                                   "definition": f"{K_BLINN_PHONG} FP32 ops per shaded fragment (Blinn-Phong "
                                                 "functor) + 9 per tested pixel; peak measured with FMA chains "
                                                 "(axr_measure_fp32_peak)"}},
        "form": {0: "persistent", 1: "phased", 2: "binned"}[info["form"]],
        "clocks": sampler.summary(),
    }
    graph.close()
    plain_graph.close()
    batch.close()
    ctx.close()
    return out, scenes


def serve_sweep(device: int, rates, seconds: float, budget_gb: float, readback: str = "colour", mix: str = "soup",
                n_assets: int = 64, seed: int = 6, overlap: bool = False) -> dict:
    """Serving loop under open-loop Poisson load: per offered rate, p50/p99 latency (arrival
    to colour read-back done, server clock) and achieved frames/s, for the batched loop and
    for the same loop rendering every request alone with the per-draw path.

    mix "soup": 90% requests of the small-triangle configuration (a 200,000-triangle soup at
    3840x2160, Gouraud, one of `n_assets` seeded soups), 10% heightfields (1920x1080,
    Blinn-Phong, random camera azimuth). mix "c4": 90% requests drawn from the mixed batch's
    per-draw distribution (a random draw of the 512-draw plan: its sphere, resolution,
    camera and texture), 10% heightfields."""
    from axiomr_gb300 import api

    rng = np.random.default_rng(seed)
    hf = W.heightfield_scene()
    if mix == "soup":
        common = [W.soup_scene(seed=1000 + k) for k in range(n_assets)]
    else:
        common = W.batch_scenes()
    gouraud, blinn = api.GouraudShader(), api.BlinnPhongShader()
    out_modes = {}
    for mode in ("batched", "per_request"):
        srv = api.Server(device, budget_bytes=int(budget_gb * (1 << 30)), max_batch=64, max_inflight=2,
                         per_request=(mode == "per_request"), overlap_kernels=overlap)
        mesh_ids = {}
        for sc in common:
            if id(sc.mesh) not in mesh_ids:
                mesh_ids[id(sc.mesh)] = srv.add_mesh(sc.mesh)
        reqs = [(mesh_ids[id(sc.mesh)], api.Camera.from_workload(sc.camera),
                 gouraud if sc.shader.kind == W.SHADER_GOURAUD else blinn, sc.width, sc.height) for sc in common]
        hf_id = srv.add_mesh(hf.mesh)
        # pinned colour buffers, reused round robin by the requests in flight
        keep = []
        lib = srv.lib
        big = max(sc.width * sc.height for sc in common)
        if readback == "colour":
            ring = [pinned_bytes(lib, big * 4, keep) for _ in range(96)]
            hf_ring = [pinned_bytes(lib, 1920 * 1080 * 4, keep) for _ in range(16)]
        elif readback == "png":  # RGB PNG files encoded on the GPU instead of the raw plane
            cap = max(api.png_bound(sc.width, sc.height, 3) for sc in common)
            ring = [pinned_bytes(lib, cap, keep) for _ in range(96)]
            hf_ring = [pinned_bytes(lib, api.png_bound(1920, 1080, 3), keep) for _ in range(16)]
        else:
            ring, hf_ring = [None], [None]

        def out(buf):
            return {"png_channels": 3, "out_png": buf} if readback == "png" else {"out_bgra": buf}

        # warm-up: every asset resident once, framebuffer pools filled, then two full-size
        # batches at once so that both in-flight slots have grown their scratch
        ts = [srv.submit(*r, **out(ring[k % len(ring)])) for k, r in enumerate(reqs)]
        ts.append(srv.submit(hf_id, api.Camera.from_workload(hf.camera), blinn, 1920, 1080, **out(hf_ring[0])))
        for t in ts:
            srv.wait(t)
        srv.hold(True)
        ts = [srv.submit(*reqs[k % len(reqs)], **out(ring[k % len(ring)])) for k in range(2 * 64 - 2)]
        ts += [srv.submit(hf_id, api.Camera.from_workload(hf.camera), blinn, 1920, 1080, **out(hf_ring[k]))
               for k in range(2)]
        srv.hold(False)
        for t in ts:
            srv.wait(t)
        per_rate = []
        for rate in rates:
            n = max(1, int(rate * seconds))
            gaps = rng.exponential(1.0 / rate, n)
            offs = (np.cumsum(gaps) * 1e9).astype(np.int64)
            kinds = rng.random(n) < 0.9
            which = rng.integers(0, len(reqs), n)
            az = rng.random(n) * 360.0
            tickets = [None] * n
            # the submitting loop must not pause: a garbage collection inside it would delay
            # submissions and show up as request latency (arrivals are scheduled, open loop)
            gc.collect()
            gc.disable()
            t0 = srv.now_ns() + 2_000_000
            k = 0
            slot = hf_slot = 0
            while k < n:
                now = srv.now_ns()
                while k < n and t0 + int(offs[k]) <= now:
                    if kinds[k]:
                        tickets[k] = srv.submit(*reqs[which[k]], arrival_ns=t0 + int(offs[k]),
                                                **out(ring[slot % len(ring)]))
                        slot += 1
                    else:
                        c = W.orbit_camera(2.5, 30.0, float(az[k]), 1920, 1080)
                        tickets[k] = srv.submit(hf_id, api.Camera.from_workload(c), blinn, 1920, 1080,
                                                arrival_ns=t0 + int(offs[k]), **out(hf_ring[hf_slot % len(hf_ring)]))
                        hf_slot += 1
                    k += 1
                if k < n:
                    wait = (t0 + int(offs[k]) - srv.now_ns()) / 1e9
                    if wait > 2e-4:
                        time.sleep(wait - 1e-4)
            gc.enable()
            lat, sizes, last, fails = [], [], 0, 0
            for t in tickets:
                r = srv.wait(t)
                if r["status"] != 0:
                    fails += 1
                    continue
                lat.append((r["done_ns"] - r["arrival_ns"]) / 1e6)
                sizes.append(r["batch_size"])
                last = max(last, r["done_ns"])
            span = (last - t0) / 1e9
            lat = np.asarray(lat)
            per_rate.append({"offered_rps": rate, "requests": n, "failed": fails,
                             "achieved_fps": round(len(lat) / span, 1) if span > 0 else None,
                             "p50_ms": round(float(np.percentile(lat, 50)), 3) if lat.size else None,
                             "p99_ms": round(float(np.percentile(lat, 99)), 3) if lat.size else None,
                             "mean_batch": round(float(np.mean(sizes)), 2) if sizes else None})
            print(json.dumps({"mix": mix, "mode": mode, **per_rate[-1]}), file=sys.stderr, flush=True)
        st = srv.stats()
        srv.close()
        for p in keep:
            lib.axr_host_free(p)
        out_modes[mode] = {"rates": per_rate, "uploads": st["uploads"], "evictions": st["evictions"],
                           "framebuffers": st["framebuffers"], "peak_resident_gb": round(st["peak_bytes"] / 2**30, 2)}
    return out_modes


def serve_scalars(modes: dict, prefix: str = "serve") -> dict:
    """Flat per-rate figures of a serving sweep (p50/p99 of both modes, achieved frames/s)."""
    out = {}
    for mode, tag in (("batched", "batched"), ("per_request", "per_req")):
        for r in modes[mode]["rates"]:
            rps = int(r["offered_rps"])
            out[f"{prefix}_{tag}_p50_ms_{rps}rps"] = r["p50_ms"]
            out[f"{prefix}_{tag}_p99_ms_{rps}rps"] = r["p99_ms"]
            out[f"{prefix}_{tag}_fps_{rps}rps"] = r["achieved_fps"]
    return out


def run_serve(args, dist: Dist):
    desc = WORKLOADS["serve"][1]
    rates = [float(r) for r in args.rates.split(",") if r]
    modes = serve_sweep(dist.local_rank, rates, args.serve_seconds, args.budget_gb, args.readback, args.serve_mix,
                        overlap=bool(args.serve_overlap))
    top = modes["batched"]["rates"][-1]
    if args.serve_mix == "c4":
        desc = desc.replace("requests of the small-triangle configuration (200,000 triangles, 3840x2160, Gouraud; "
                            "one of 64 seeded soups)", "requests drawn from the mixed batch's per-draw distribution")
    return {
        "metric": "frames/s", "value": top["achieved_fps"], "unit": "frames/s", "n_gpus": dist.world,
        "steps": len(rates), "warmup": 1, "ms_per_step": None, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded generators in axiomr_gb300/workloads.py)",
        "config": {"workload": f"serve: {desc}", "seconds_per_rate": args.serve_seconds, "max_batch": 64,
                   "max_inflight": 2, "overlap_kernels": bool(args.serve_overlap), "budget_gb": args.budget_gb,
                   "readback": args.readback, "mix": args.serve_mix},
        "serving": modes,
    }


def cpu_batch_sample(scenes, budget_s: float, steps: int):
    """The CPU restatement of the reference pipeline (oracle/port) on every 32nd draw of the
    mixed batch, all host threads; frames/s over those draws (clears included, as the
    reference renderer's frame). The `cpu_baseline` figure of our arm's line: a bounded
    sample, so that the GPU run stays short."""
    from oracle import Oracle

    port = Oracle("port")
    threads = os.cpu_count() or 1
    sample = scenes[:: max(1, len(scenes) // BATCH_REF_SAMPLE)][:BATCH_REF_SAMPLE]
    vps = [port.camera(sc.camera)[2] for sc in sample]

    def step():
        for sc, vp in zip(sample, vps):
            port.draw(sc, vp, threads=threads)

    t0 = time.perf_counter()
    step()  # warm-up, also sizes the run
    t1 = time.perf_counter() - t0
    reps = max(1, min(steps, int(budget_s / max(t1, 1e-6))))
    times = []
    for _ in range(reps):
        t = time.perf_counter()
        step()
        times.append(time.perf_counter() - t)
    value = len(sample) * len(times) / sum(times)
    return value, threads, times, (f"{reps} x {len(sample)} draws (every {len(scenes) // len(sample)}th draw of the "
                                   f"batch) on {threads} host threads ({os.uname().machine})")


def run_reference(args, dist: Dist):
    make, desc = WORKLOADS[args.workload]
    if args.workload == "batch":
        # every step renders every draw of the batch (the same configuration as our arm),
        # with the same warm-up and step counts
        from oracle import Oracle

        scenes = W.batch_scenes(count=args.draws, resolution_scale=args.scale)
        port = Oracle("port")
        threads = os.cpu_count() or 1
        vps = [port.camera(sc.camera)[2] for sc in scenes]

        def step():
            for sc, vp in zip(scenes, vps):
                port.draw(sc, vp, threads=threads)

        for _ in range(args.warmup):
            step()
        times = []
        for _ in range(args.steps):
            t = time.perf_counter()
            step()
            times.append(time.perf_counter() - t)
        value = len(scenes) * len(times) / sum(times)
        sample = (f"{args.steps} steps of all {len(scenes)} draws after {args.warmup} warm-up steps, one drawMesh "
                  f"per draw (clears included), on {threads} host threads ({os.uname().machine})")
        return {
            "metric": "frames/s", "value": round(value, 4), "unit": "frames/s", "n_gpus": dist.world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1e3 * sum(times) / len(times), 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded generators in axiomr_gb300/workloads.py)",
            "config": batch_config(args, dist, len(scenes)),
            "form_desc": "reference CPU TiledPipeline (C restatement in oracle/port), one drawMesh per draw",
            "impl": "reference",
            "cpu_baseline": {"value": round(value, 4), "unit": "frames/s", "cores": threads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": round(value, 4), "unit": "frames/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        }
    scene = make() if make is not None else W.soup_scene(seed=1000)  # serve: one request of the common kind
    from oracle import Oracle

    port = Oracle("port")
    threads = os.cpu_count() or 1
    vp = port.camera(scene.camera)[2]
    t0 = time.perf_counter()
    port.draw(scene, vp, threads=threads)
    t1 = time.perf_counter() - t0
    for _ in range(max(0, min(args.warmup, int(10.0 / max(t1, 1e-6))) - 1)):
        port.draw(scene, vp, threads=threads)
    # each step is one full frame; if K frames would exceed ~3 minutes, a step renders
    # a contiguous fraction of the faces and counts as that fraction of a frame
    frac = min(1.0, 180.0 / max(1e-9, args.steps * t1))
    if frac < 1.0:
        import dataclasses

        nf = max(1, int(scene.mesh.num_faces * frac))
        frac = nf / scene.mesh.num_faces
        scene = dataclasses.replace(scene, mesh=dataclasses.replace(scene.mesh, groups=np.asarray(
            [[0, nf, 0]], np.uint32)))
    times = []
    for _ in range(args.steps):
        t = time.perf_counter()
        port.draw(scene, vp, threads=threads)
        times.append(time.perf_counter() - t)
    value = frac * len(times) / sum(times)
    sample = (f"{args.steps} steps, each {'a full frame' if frac >= 1.0 else f'{frac:.3f} of a frame'} "
              f"of the workload on {threads} host threads ({os.uname().machine})")
    return {
        "metric": "frames/s", "value": round(value, 4), "unit": "frames/s", "n_gpus": dist.world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1e3 * sum(times) / len(times), 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded generators in axiomr_gb300/workloads.py)",
        "config": {"workload": f"{args.workload}: {desc}", "form": "reference CPU TiledPipeline (C restatement)"},
        "impl": "reference",
        "cpu_baseline": {"value": round(value, 4), "unit": "frames/s", "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": round(value, 4), "unit": "frames/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main():
    args = parse_args()
    dist = Dist()
    try:
        if args.impl == "reference":
            if dist.rank == 0:
                print(json.dumps(run_reference(args, dist)), flush=True)
            return
        if args.workload == "serve":
            out = run_serve(args, dist)
            if dist.rank == 0:
                print(json.dumps(out), flush=True)
            return
        if args.workload == "batch":
            out, scenes = run_batch(args, dist)
            if args.brief_serve_seconds > 0 and args.draws == 512 and args.scale == 1.0:
                # a short serving sweep (the metric's p50/p99 request latency per offered
                # load), its flat figures kept beside the end-to-end number
                rates = [float(r) for r in args.rates.split(",") if r]
                modes = serve_sweep(dist.local_rank, rates, args.brief_serve_seconds, args.budget_gb, "colour",
                                    "soup", n_assets=16)
                out["serving"] = {"mix": "soup", "seconds_per_rate": args.brief_serve_seconds, "assets": 16,
                                  "modes": modes}
                out["e2e"].update(serve_scalars(modes))
            if dist.rank == 0 and dist.world == 1 and not args.no_cpu_baseline:
                value, threads, times, sample = cpu_batch_sample(scenes, args.cpu_budget_s, args.steps)
                out["cpu_baseline"] = {"value": round(value, 4), "unit": "frames/s", "cores": threads,
                                       "kind": "port", "sample": sample}
            if dist.rank == 0:
                print(json.dumps(out), flush=True)
            return
        out, scene = run_ours(args, dist)
        if dist.rank == 0:
            if dist.world == 1 and not args.no_cpu_baseline:
                out["cpu_baseline"] = cpu_baseline(scene, args.steps, args.cpu_budget_s)
            print(json.dumps(out), flush=True)
    finally:
        dist.close()


if __name__ == "__main__":
    main()
