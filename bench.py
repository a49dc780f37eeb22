#!/usr/bin/env python3
"""Throughput benchmark of the GB300 DFPSR triangle path.

One step renders one frame of the workload (default: the 1920x1080 terrain, a
512x512 height grid of 522k triangles with a 1024x1024 mip-mapped texture and
texture x vertex-colour shading, depth tested) through dsrg_model_render.

  value  fragments/s with the colour and depth targets resident in HBM, CUDA events
         on the renderer's stream around each frame, L2 flushed before every frame.
  e2e    the same through the C ABI with page-locked HOST images, wall clock around each
         call: the library draws them in place through their device addresses, so the
         tile pass reads the depth image and writes colour and depth over NVLink-C2C
         inside the timed region (no staging copies).

`python bench.py --impl reference` times the reference's CPU renderer on this
host's cores instead (the reference built from source where available, otherwise
the oracle's C restatement of it).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Mfrag/s & frames/s plain vs batched; fwd+bwd views/s at grad rel err ≤1e-3"
BYTES_PER_FRAGMENT = 28  # depth read + depth write + colour write + 4 bilinear RGBA8 texels


def parse_args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--workload", choices=["terrain", "random"], default="terrain")
    p.add_argument("--cpu-seconds", type=float, default=12.0, help="bound of the CPU-baseline sample")
    p.add_argument("--batch-frames", type=int, default=256, help="frames of the mixed-size batch (0 skips it)")
    p.add_argument("--diff-views", type=int, default=64, help="views of the differentiable render (0 skips it)")
    p.add_argument("--light-sprites", type=int, default=4096, help="sprites of the deferred-light pass (0 skips it)")
    p.add_argument("--c0", type=int, default=1, help="also measure the 800x600 random-triangle workload (0 skips it)")
    p.add_argument("--shadow-tuning", default="auto",
                   help="the light pass's shadow batch: auto (the autotuner on that batch) or TxCxRxWxM like --tuning")
    p.add_argument("--tuning", default="auto",
                   help="tile kernel launch shape THREADSxCTAS_PER_SMxSMALL_ROWSxSMALL_WIDTH[xRESOLVE] (e.g. 128x8x8x16x1), or auto")
    return p.parse_args()


def workload(name, world: int = 1):
    """The scene of a plain workload and its config, the same for both arms of the benchmark."""
    from dfpsr_gb300 import scenes
    if name == "terrain":
        s = scenes.terrain(seed=1234)
        cfg = {"workload": "terrain 1920x1080, 512x512 height grid (522,242 triangles), 1024x1024 RGBA8 texture with mips, "
                           "texture x vertex colour, depth tested", "width": 1920, "height": 1080,
               "triangles": s.triangle_count, "seed": 1234}
    else:
        s = scenes.random_triangles(seed=1234)
        cfg = {"workload": "800x600, 20,000 random triangles, 256x256 RGBA8 texture with mips, vertex colour x texture, "
                           "depth tested", "width": 800, "height": 600, "triangles": s.triangle_count, "seed": 1234}
    cfg["l2"] = "flushed before every GPU frame (256 MB write)"
    cfg["parallelism"] = f"replicas ({world} GPUs)" if world > 1 else "single GPU"
    return s, cfg


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0}, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""

    FIELDS = "index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown," \
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap"

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.file = None

    def __enter__(self):
        try:
            fd, self.file = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            # nvidia-smi appends to its own descriptor; the readers below open the file separately, so
            # reading never moves the writer's offset
            self.sink = open(self.file, "a")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=self.sink, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def _lines(self):
        try:
            with open(self.file) as f:
                return f.read().splitlines()
        except Exception:
            return []

    def count(self) -> int:
        if not self.file:
            return 0
        return sum(1 for line in self._lines() if line.count(",") >= 8)

    def wait_first(self, timeout: float = 5.0):
        """Waits until nvidia-smi has written its first sample (it takes a moment to start)."""
        t0 = time.perf_counter()
        while self.proc and self.count() < 1 and time.perf_counter() - t0 < timeout:
            time.sleep(0.02)

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.sink.close()

    def summary(self):
        if not self.proc or not self.file:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        lines = self._lines()
        try:
            os.unlink(self.file)
        except Exception:
            pass
        for line in lines:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower() in ("active", "1"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def batched_section(ctx, args, flush):
    """The mixed-size batch: 256 frames of random triangles (resolutions uniform over 64x64,
    256x256, 640x480 and 1024x768, 1k-200k triangles log-uniform, a 256x256 texture each),
    drawn per frame through dsrg_model_render (plain) and all at once through dsrg_batch_render
    (batched, after the autotuner picked the tile kernel's launch shape), targets in HBM."""
    import torch
    import dfpsr_gb300 as d
    from dfpsr_gb300 import scenes
    frames = scenes.batch_frames(seed=4321, frames=args.batch_frames)
    stream = torch.cuda.ExternalStream(ctx.stream)
    models = [d.Model(ctx, s) for s in frames]
    colors = [torch.zeros((s.height, s.width), dtype=torch.int32, device="cuda") for s in frames]
    depths = [torch.zeros((s.height, s.width), dtype=torch.float32, device="cuda") for s in frames]
    batch = d.Batch(ctx)
    for i, m in enumerate(models):
        batch.add_frame(colors[i], depths[i])
        batch.give_task(i, m)

    def clear():
        with torch.cuda.stream(stream):
            flush.fill_(1.0)
            for c, z in zip(colors, depths):
                c.zero_()
                z.zero_()

    tuning = batch.autotune(rounds=3)
    ctx.set_counting(True)
    clear()
    batch.render()
    stats = ctx.stats()
    fragments = stats["fragments"]
    ctx.set_counting(False)
    for _ in range(3):
        clear()
        batch.render()
    steps = max(1, min(args.steps, 10))
    batch_ms, raster_ms = [], []
    for _ in range(steps):
        clear()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        batch.render()
        b.record(stream)
        raster_ms.append(ctx.stats()["raster_milliseconds"])
        batch_ms.append((a, b))
    torch.cuda.synchronize()
    batch_s = statistics.median([a.elapsed_time(b) for a, b in batch_ms]) / 1e3

    def plain_pass():
        total = 0.0
        for i, m in enumerate(models):
            with torch.cuda.stream(stream):
                flush.fill_(1.0)
                colors[i].zero_()
                depths[i].zero_()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            ctx.render(m, m.camera, colors[i], depths[i])
            b.record(stream)
            b.synchronize()
            total += a.elapsed_time(b) / 1e3
        return total

    plain_pass()
    plain_s = min(plain_pass() for _ in range(2))
    # end to end: host images (page-locked) through the batch API
    host = [(torch.zeros((s.height, s.width), dtype=torch.int32).pin_memory().numpy(),
             torch.zeros((s.height, s.width), dtype=torch.float32).pin_memory().numpy()) for s in frames]
    hbatch = d.Batch(ctx)
    for i, m in enumerate(models):
        hbatch.add_frame(*host[i])
        hbatch.give_task(i, m)
    hbatch.render()
    e2e = []
    for _ in range(steps):
        for c, z in host:
            c.fill(0)
            z.fill(0.0)
        t0 = time.perf_counter()
        hbatch.render()
        e2e.append(time.perf_counter() - t0)
    e2e_s = statistics.median(e2e)
    host_bytes = int(sum(c.nbytes + z.nbytes for c, z in host))
    n = len(frames)
    out = {
        "workload": f"{n} frames, resolutions uniform over 64x64/256x256/640x480/1024x768, 1k-200k random triangles "
                    "(log-uniform) per frame, own 256x256 RGBA8 texture per frame, depth tested",
        "frames": n, "triangles": int(sum(s.triangle_count for s in frames)),
        "pixels": int(sum(s.width * s.height for s in frames)), "fragments": fragments,
        "draw_records": stats["draw_records"], "bin_entries": stats["bin_entries"],
        "batched": {"frames_per_s": n / batch_s, "Mfrag_per_s": fragments / batch_s / 1e6, "ms_per_batch": batch_s * 1e3,
                    "raster_ms": statistics.median(raster_ms)},
        "plain": {"frames_per_s": n / plain_s, "Mfrag_per_s": fragments / plain_s / 1e6, "ms_per_batch": plain_s * 1e3},
        "batched_over_plain": plain_s / batch_s,
        "e2e": {"frames_per_s": n / e2e_s, "Mfrag_per_s": fragments / e2e_s / 1e6,
                "h2d_bytes_per_batch": int(sum(z.nbytes for _, z in host)), "d2h_bytes_per_batch": host_bytes,
                "transfer": "in place (page-locked host images read and written through their device addresses)"},
        "tuning": tuning,
        "l2": "flushed before every batch and before every plain frame (256 MB write)",
    }
    hbatch.destroy()
    batch.destroy()
    for m in models:
        m.destroy()
    return out


def diff_section(ctx, args):
    """Differentiable rendering: 64 views 256x256 of a 50,000-triangle torus into float RGBA
    targets, parameters a 512x512 float RGBA texture, per-point colours and a directional light;
    one step = forward (with visibility buffer) + L2 loss against images rendered from
    parameters perturbed by N(0, 0.05) + the hand-written adjoint.  The gradient is checked
    against the FP64 host oracle, whose time is reported as a CPU figure (not a reference
    baseline: the reference has no differentiable renderer)."""
    import torch
    import dfpsr_gb300 as d
    from dfpsr_gb300 import scenes
    problem = scenes.diff_problem(seed=99, views=args.diff_views, size=256, texture_size=512)
    model = d.Model(ctx, problem.mesh)
    renderer = d.Diff(ctx, model, 512, 512, problem.ambient)
    cams = []
    for loc in problem.cameras:
        cam = d.camera_struct(problem.mesh)
        for i in range(12):
            cam.location[i] = float(loc[i])
        cams.append(cam)
    views, h, w = len(cams), problem.height, problem.width
    dev = lambda a: torch.tensor(np.ascontiguousarray(a), device="cuda")
    params = [dev(problem.texture), dev(problem.vertex_colors), dev(problem.light)]
    target_params = [dev(problem.target_texture), dev(problem.target_vertex_colors), dev(problem.target_light)]
    images = torch.empty((views, h, w, 4), device="cuda")
    targets = torch.empty_like(images)
    vis = torch.empty((views, h, w, 3), dtype=torch.int32, device="cuda")
    tvis = torch.empty_like(vis)
    grad = torch.empty_like(images)
    loss = torch.empty(1, device="cuda")
    grads = [torch.empty_like(p) for p in params]
    transform = problem.mesh.model_to_world
    renderer.forward(cams, transform, *target_params, targets, tvis)

    def step(deterministic):
        renderer.forward(cams, transform, *params, images, vis)
        renderer.l2_loss(images, targets, grad, loss)
        renderer.adjoint(views, w, h, transform, *params, vis, grad, *grads, deterministic)

    out = {"workload": f"{views} views {w}x{h} of a {problem.mesh.triangle_count}-triangle torus, float RGBA targets, "
                       "parameters 512x512 float RGBA texture + per-point colours + directional light, L2 loss against "
                       "images from parameters perturbed by N(0, 0.05)"}
    # the tile shape for this workload: a few candidates timed on the step itself, the fastest kept
    before = ctx.tuning()
    best = None
    for shape in ((128, 8, 8, 16), (256, 4, 8, 16), (256, 4, 0, 0)):
        ctx.set_tuning(threads_per_tile=shape[0], ctas_per_sm=shape[1], small_rows=shape[2], small_width=shape[3], resolve=1)
        step(False)
        t0 = time.perf_counter()
        for _ in range(3):
            step(False)
        dt = time.perf_counter() - t0
        if best is None or dt < best[0]:
            best = (dt, ctx.tuning())
    ctx.set_tuning(**best[1])
    out["tuning"] = best[1]
    steps = max(1, min(args.steps, 10))
    for mode, deterministic in (("atomic", False), ("deterministic", True)):
        for _ in range(3):
            step(deterministic)
        launches0 = ctx.stats()["kernel_launches"]
        t0 = time.perf_counter()
        for _ in range(steps):
            step(deterministic)
        dt = (time.perf_counter() - t0) / steps
        out[mode] = {"views_per_s": views / dt, "ms_per_step": dt * 1e3,
                     "launches_per_step": (ctx.stats()["kernel_launches"] - launches0) / steps}
    ctx.set_tuning(**before)
    # the gradient against the FP64 host oracle, at the GPU's visibility
    from oracle import diff64
    t0 = time.perf_counter()
    shading = diff64.Shading(problem.mesh, vis.cpu().numpy().view(np.uint32), problem.texture.shape)
    g64 = shading.gradients(problem.texture, problem.vertex_colors, problem.light, problem.ambient,
                            diff64.l2_grad(images.cpu().numpy(), targets.cpu().numpy()))
    host_s = time.perf_counter() - t0
    errors = {}
    for deterministic in (False, True):
        step(deterministic)
        for name, got, want in zip(("texture", "vertex_colors", "light"), grads, g64):
            errors[f"{'deterministic' if deterministic else 'atomic'}_{name}"] = diff64.relative_error(got.cpu().numpy(), want)
    out["grad_rel_err"] = errors
    out["grad_rel_err_max"] = max(errors.values())
    out["loss"] = float(loss.item())
    out["fp64_host_oracle"] = {"seconds_per_step": host_s, "views_per_s": views / host_s, "cores": 1,
                               "kind": "FP64 numpy re-shade and gradient at fixed visibility (not a reference baseline)"}
    renderer.destroy()
    model.destroy()
    return out


def light_section(ctx, args):
    """Isometric deferred-light pass at 1920x1080: 4096 sprites 64x64 drawn with draw_higher into
    diffuse, normal and height images, 16 point lights (radius 100-400 px) each with a 6 x 512 x 512
    shadow cube map rendered from a 2,000-triangle caster model (one depth-only batch of 96 faces),
    a directed light, the point lights, blendLight.  One frame is one dsrg_sprite_frame call, timed
    with CUDA events on the library's stream.  The CPU figure is the oracle's C restatement of the
    same pass (the 96 shadow faces on every host core, the sprites and lights on one), whose output
    the GPU's must equal."""
    import torch
    import dfpsr_gb300 as d
    from dfpsr_gb300 import scenes
    from dfpsr_gb300.sprite_pass import DeferredLightPass
    m, _ = d.ortho_view(-0.7, 64, 0).arrays()
    scene = scenes.light_scene(seed=2024, sprites=args.light_sprites, light_space=(m[9:18], m[0:9]))
    threads = os.cpu_count() or 1
    gpu = DeferredLightPass(ctx, scene, threads)
    # the shadow batch's own tile-kernel shape, chosen by the autotuner on it (the context's stays)
    if args.shadow_tuning == "auto":
        shadow_tuning = gpu.tune_shadows(rounds=2)
    else:  # a given shape (profiling runs keep the autotuner's trial launches out of the launch list)
        fields = [int(v) for v in args.shadow_tuning.split("x")]
        shadow_tuning = dict(ctx.tuning(), threads_per_tile=fields[0], ctas_per_sm=fields[1], small_rows=fields[2],
                             small_width=fields[3], resolve=fields[4] if len(fields) > 4 else 1)
        gpu.shadows.set_tuning(shadow_tuning)
    stream = torch.cuda.ExternalStream(ctx.stream)
    steps = max(1, min(args.steps, 20))

    def timed(frame):
        for _ in range(3):
            frame()
        out = []
        for _ in range(steps):
            torch.cuda.synchronize()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)  # every step of the frame runs on the library's stream
            frame()
            b.record(stream)
            b.synchronize()
            out.append(a.elapsed_time(b))
        return statistics.median(out)

    ms = timed(gpu.run)  # dsrg_sprite_frame: one call
    ms_steps = timed(gpu.run_steps)  # the same frame as one call per step
    # the point-light pass alone: 20 B per lit pixel and light (normal, height, light read + write, shadow sample)
    bounds = 0
    from oracle import port, light_pass
    view = port.ortho_view(scene.camera_tilt, scene.pixels_per_tile, scene.view_index)
    for l in scene.lights:
        b = port.point_light_bound(view, scene.center, scene.width, scene.height, l["position"], l["radius"])
        if b is not None:
            bounds += int((b[2] - b[0]) * (b[3] - b[1]))
    lt = []
    for _ in range(steps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        ctx.light_points(gpu.view, scene.center, gpu.light, gpu.normal, gpu.height, gpu.light_list, threads)
        b.record(stream)
        b.synchronize()
        lt.append(a.elapsed_time(b))
    t0 = time.perf_counter()
    out, *_ = light_pass.run(scene, threads, workers=threads)
    cpu_s = time.perf_counter() - t0
    got = gpu.run().cpu().numpy().view(np.uint32)
    result = {"workload": "isometric deferred-light pass 1920x1080: 4096 sprites 64x64 (draw_higher), 16 point lights "
                          "radius 100-400 px with 6x512x512 shadow cube maps from a 2,000-triangle caster (depth-only "
                          "batch of 96 faces), directed light, blendLight",
              "frames_per_s": 1e3 / ms, "ms_per_frame": ms,
              "frame_call": "dsrg_sprite_frame: every step on the library's stream, a host wait inside the shadow batch "
                            "and one at the end; CUDA events on that stream",
              "ms_per_frame_one_call_per_step": ms_steps,
              "shadow_batch_tuning": "{threads_per_tile}x{ctas_per_sm}x{small_rows}x{small_width}x{resolve}".format(**shadow_tuning),
              "point_lights_ms": statistics.median(lt), "lit_pixel_lights": bounds,
              "point_lights_GB_per_s": 20.0 * bounds / (statistics.median(lt) / 1e3) / 1e9,
              "parity_with_oracle": bool(np.array_equal(got, out)),
              "cpu_oracle": {"frames_per_s": 1.0 / cpu_s, "cores": threads, "kind": "port",
                             "sample": f"one frame of the same pass, oracle C restatement: the 96 shadow faces on {threads} "
                                       "threads, the sprites and lights on one"}}
    gpu.destroy()
    result["dense_models"] = dense_models_section(ctx)
    return result


def dense_models_section(ctx, instances: int = 64):
    """The sprite world's model instances (drawModel: renderDenseModel, low quality) at 1920x1080:
    `instances` placements of a 3,200-triangle vertex-coloured torus drawn one after another into
    the height, diffuse and normal images, timed with CUDA events; the images must equal the
    oracle's after the whole sequence."""
    import torch
    import dfpsr_gb300 as d
    from dfpsr_gb300 import scenes
    from oracle import port
    sc = scenes.dense_scene(seed=77, width=1920, height=1080, major=80, minor=20, pixels_per_tile=64)
    rng = np.random.default_rng(5)
    places = [((float(rng.uniform(0, 1920)), float(rng.uniform(0, 1080))),
               np.concatenate([rng.uniform(-1, 1, 3), scenes.random_rotation(rng).reshape(-1)]).astype(np.float32))
              for _ in range(instances)]
    model = d.DenseModel(ctx, sc.positions, sc.polygons, sc.colors)
    view = d.ortho_view(sc.camera_tilt, sc.pixels_per_tile, sc.view_index)
    stream = torch.cuda.ExternalStream(ctx.stream)
    h = torch.tensor(sc.height, device="cuda")
    di = torch.zeros((1080, 1920), dtype=torch.int32, device="cuda")
    n = torch.zeros_like(di)

    def run():
        h.copy_(torch.tensor(sc.height, device="cuda"))
        di.zero_()
        n.zero_()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for origin, transform in places:
            ctx.dense_render(model, view, h, di, n, origin, transform, False)
        b.record(stream)
        b.synchronize()
        return a.elapsed_time(b)

    run()
    ms = statistics.median([run() for _ in range(5)])
    calls = {"h": h.clone(), "d": di.clone(), "n": n.clone()}

    def run_many():
        h.copy_(torch.tensor(sc.height, device="cuda"))
        di.zero_()
        n.zero_()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        ctx.dense_render_many([(model, origin, transform) for origin, transform in places], view, h, di, n, False)
        b.record(stream)
        b.synchronize()
        return a.elapsed_time(b)

    run_many()
    ms_many = statistics.median([run_many() for _ in range(5)])
    same_calls = bool(torch.equal(calls["h"], h) and torch.equal(calls["d"], di) and torch.equal(calls["n"], n))
    tris = port.dense_model(sc.positions, sc.polygons, sc.colors)
    pv = port.ortho_view(sc.camera_tilt, sc.pixels_per_tile, sc.view_index)
    rh, rd, rn = sc.height, np.zeros((1080, 1920), np.uint32), np.zeros((1080, 1920), np.uint32)
    t0 = time.perf_counter()
    for origin, transform in places:
        rh, rd, rn = port.dense_render(tris, pv, rh, rd, rn, origin, transform, False)
    cpu_s = time.perf_counter() - t0
    same = (np.array_equal(h.cpu().numpy().view(np.uint32), rh.view(np.uint32)) and
            np.array_equal(di.cpu().numpy().view(np.uint32), rd) and np.array_equal(n.cpu().numpy().view(np.uint32), rn))
    model.destroy()
    count = len(tris)
    return {"workload": f"{instances} instances of a {count}-triangle dense torus at 1920x1080 (renderDenseModel, low quality)",
            "one_call_per_instance": {"ms_per_sequence": ms, "instances_per_s": instances / (ms / 1e3)},
            "ms_per_sequence": ms_many, "instances_per_s": instances / (ms_many / 1e3),
            "triangles_per_s": instances * count / (ms_many / 1e3), "parity_with_oracle": bool(same),
            "one_call_equals_calls": same_calls,
            "cpu_oracle": {"instances_per_s": instances / cpu_s, "cores": 1, "kind": "port",
                           "sample": "the same sequence, oracle C restatement, one thread"}}


def cpu_baseline(scene, seconds: float):
    """The oracle's C restatement of the reference renderer on all host cores (band split like
    renderer_end, CommandQueue::execute with 12 bands), over a bounded number of frames."""
    from oracle import port
    threads = os.cpu_count() or 1
    pm = port.PreparedModel(scene)
    _, _, info = port.render(scene, bands=12, threads=threads, prepared=pm)
    frames, t0 = 0, time.perf_counter()
    while True:
        port.render(scene, bands=12, threads=threads, prepared=pm)
        frames += 1
        if time.perf_counter() - t0 > seconds or frames >= 50:
            break
    dt = (time.perf_counter() - t0) / frames
    return {"value": info["fragments"] / dt / 1e6, "unit": "Mfrag/s", "cores": min(threads, 12), "kind": "port",
            "sample": f"{frames} frame(s) of the same workload, oracle C port, 12 row bands on {min(threads, 12)} threads",
            "frames_per_s": 1.0 / dt}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    scene, cfg = workload(args.workload, int(os.environ.get("WORLD_SIZE", "1")))
    from oracle import port, ref
    threads = os.cpu_count() or 1
    use_ref = ref.available("shipped")
    if use_ref:
        model = ref.RefModel(scene, "shipped")
        frame = lambda: model.render(threaded=True)
        kind, sample = "reference", "reference renderer_begin/giveTask/end (as shipped, -O2 -march=native), threaded bands"
    else:
        pm = port.PreparedModel(scene)
        frame = lambda: port.render(scene, bands=12, threads=threads, prepared=pm)
        kind, sample = "port", "oracle C port of the reference renderer, 12 row bands"
    _, _, info = port.render(scene)
    fragments = info["fragments"]
    for _ in range(max(1, min(args.warmup, 2))):
        frame()
    times = []
    budget = time.perf_counter()
    for _ in range(args.steps):
        t0 = time.perf_counter()
        frame()
        times.append(time.perf_counter() - t0)
        if time.perf_counter() - budget > 120:
            break
    dt = sum(times) / len(times)
    value = fragments / dt / 1e6
    cores = min(threads - 1 if use_ref else threads, 12) or 1
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "Mfrag/s", "n_gpus": args.gpus,
            "steps": len(times), "warmup": args.warmup, "ms_per_step": dt * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32+int64", "data": "synthetic (seeded)", "config": cfg,
            "frames_per_s": 1.0 / dt,
            "cpu_baseline": {"value": value, "unit": "Mfrag/s", "cores": cores, "kind": kind, "sample": sample},
            "e2e": {"value": value, "unit": "Mfrag/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    sys.stderr.flush()
    if use_ref:
        # the reference library's own heap bookkeeping reports spuriously when Python tears it down
        os._exit(0)


def plain_record(ctx, scene, cfg, args, flush, dist, world, local, workload_key, with_cpu):
    """One plain workload through dsrg_model_render: fragments/s with the targets in HBM (CUDA
    events on the renderer's stream, L2 flushed before every frame), the same end to end with
    page-locked host images, the tile pass's roofline and the CPU baseline."""
    import torch
    import dfpsr_gb300 as d
    from dfpsr_gb300 import replicas
    h, w = scene.height, scene.width
    model = d.Model(ctx, scene)
    # the model's device arrays, which a frame reads at least once: positions (12 B per point),
    # polygon indices (16 B), corner colours and texture coordinates (2 x 64 B per polygon) and
    # the fan table (4 B per fan triangle)
    model_bytes = (12 * int(np.asarray(scene.positions).shape[0]) + (16 + 128) * int(np.asarray(scene.poly_indices).shape[0])
                   + 4 * int(scene.triangle_count))
    stream = torch.cuda.ExternalStream(ctx.stream)
    color = torch.zeros((h, w), dtype=torch.int32, device="cuda")
    depth = torch.zeros((h, w), dtype=torch.float32, device="cuda")

    # the tile kernel's launch shape for this workload, chosen by the library's autotuner on a
    # one-frame batch of it (the plain path below uses the context's tuning)
    if args.tuning == "auto":
        tune_batch = ctx.batch()
        tune_batch.add_frame(color, depth)
        tune_batch.give_task(0, model)
        tuning = tune_batch.autotune(rounds=3)
        tune_batch.destroy()
    else:  # a given shape (profiling runs keep the autotuner's trial launches out of the launch list)
        fields = [int(v) for v in args.tuning.split("x")]
        ctx.set_tuning(threads_per_tile=fields[0], ctas_per_sm=fields[1], small_rows=fields[2], small_width=fields[3],
                       resolve=fields[4] if len(fields) > 4 else 0)
        tuning = ctx.tuning()

    # fragments per frame before the depth test: deterministic, counted once by the kernels themselves
    ctx.set_counting(True)
    ctx.render(model, model.camera, color, depth)
    frame_stats = ctx.stats()
    fragments = frame_stats["fragments"]
    ctx.set_counting(False)

    def frame_device():
        with torch.cuda.stream(stream):
            flush.fill_(1.0)
            color.zero_()
            depth.zero_()
        start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        start.record(stream)
        ctx.render(model, model.camera, color, depth)
        stop.record(stream)
        return start, stop

    for _ in range(args.warmup):
        frame_device()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    events, raster_ms = [], []
    with ClockSampler(local) as clocks:
        clocks.wait_first()
        launches0 = ctx.stats()["kernel_launches"]
        walked0 = ctx.walked_fragments()
        for _ in range(args.steps):
            events.append(frame_device())
            raster_ms.append(ctx.stats()["raster_milliseconds"])
        torch.cuda.synchronize()
        # fragments the timed frames depth-tested (early culling on): the work actually walked
        walked = (ctx.walked_fragments() - walked0) / args.steps
        launches = ctx.stats()["kernel_launches"] - launches0
        # the timed region can be shorter than the sampling period: keep the same load (untimed)
        # until a few samples under load exist
        t0 = time.perf_counter()
        while clocks.count() < 4 and time.perf_counter() - t0 < 3.0:
            frame_device()
        torch.cuda.synchronize()
    step_ms = [a.elapsed_time(b) for a, b in events]
    total_s = replicas.max_over_ranks(sum(step_ms) / 1e3, dist)
    if dist:
        dist.barrier()

    # end to end through the C ABI with page-locked host images
    host_color = torch.zeros((h, w), dtype=torch.int32).pin_memory().numpy()
    host_depth = torch.zeros((h, w), dtype=torch.float32).pin_memory().numpy()
    for _ in range(max(1, args.warmup // 2)):
        ctx.render(model, model.camera, host_color, host_depth)
    e2e_times = []
    for _ in range(args.steps):
        host_color.fill(0)
        host_depth.fill(0.0)
        t0 = time.perf_counter()
        ctx.render(model, model.camera, host_color, host_depth)
        e2e_times.append(time.perf_counter() - t0)
    e2e_s = replicas.max_over_ranks(sum(e2e_times), dist)
    model.destroy()

    peaks, peak_kind = measured_peaks()
    raster_avg_s = (sum(raster_ms) / len(raster_ms)) / 1e3
    peak = float(peaks.get("hbm_gbs", 6800.0))
    achieved = BYTES_PER_FRAGMENT * walked / raster_avg_s / 1e9
    achieved_counted = BYTES_PER_FRAGMENT * fragments / raster_avg_s / 1e9
    traffic = None
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
            traffic = json.load(f).get(workload_key)
    except Exception:
        pass
    rec = {
        "value": world * fragments * args.steps / total_s / 1e6, "unit": "Mfrag/s",
        "ms_per_step": total_s * 1e3 / args.steps,
        "frames_per_s": world * args.steps / total_s,
        "fragments_per_frame": fragments,
        "walked_fragments_per_frame": walked,
        "frame_stats": {"draw_records": frame_stats["draw_records"], "bin_entries": frame_stats["bin_entries"]},
        "e2e": {"value": world * fragments * args.steps / e2e_s / 1e6, "unit": "Mfrag/s",
                "h2d_bytes_per_step": int(host_depth.nbytes),
                "d2h_bytes_per_step": int(host_color.nbytes + host_depth.nbytes),
                "frames_per_s": world * args.steps / e2e_s,
                "transfer": "in place: the tile pass reads the host depth image and writes the host colour and "
                            "depth images through their device addresses (page-locked memory over NVLink-C2C)"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_source": peak_kind, "traffic": traffic, "kernel": "raster_kernel (tile pass with the fused resolve)",
                     "kernel_ms": raster_avg_s * 1e3, "algorithmic_bytes_per_launch": BYTES_PER_FRAGMENT * walked,
                     "model": "28 B per walked fragment (depth read + depth write + colour write + 4 RGBA8 texels); walked = "
                              "fragments the timed frames depth-tested, after early depth culling",
                     "pre_depth_test": {"achieved": achieved_counted, "frac": achieved_counted / peak,
                                        "algorithmic_bytes_per_launch": BYTES_PER_FRAGMENT * fragments,
                                        "note": "28 B per fragment counted before the depth test (the metric's unit); early "
                                                "culling never walks most of them on high-overdraw scenes, so this can exceed 1"}},
        "frame_roofline": {"bound": "hbm", "unit": "GB/s", "peak": peak, "peak_source": peak_kind,
                           "algorithmic_bytes": model_bytes + BYTES_PER_FRAGMENT * walked,
                           "achieved": (model_bytes + BYTES_PER_FRAGMENT * walked) / (total_s / args.steps) / 1e9,
                           "frac": (model_bytes + BYTES_PER_FRAGMENT * walked) / (total_s / args.steps) / 1e9 / peak,
                           "model": "the whole frame: the model's device arrays read once (positions, polygon indices, corner "
                                    "colours and texture coordinates, fan table) plus 28 B per walked fragment, over the "
                                    "frame's CUDA-event time"},
        "gpu_launches": launches,
        "tuning": tuning,
        "clocks": clocks.summary(),
    }
    if with_cpu:
        rec["cpu_baseline"] = cpu_baseline(scene, args.cpu_seconds)
    return rec


def main():
    args = parse_args()
    if args.impl == "reference":
        run_reference(args)
        return
    import torch
    import dfpsr_gb300 as d

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    scene, cfg = workload(args.workload, world)
    ctx = d.Context(local)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")  # > 129 MB of L2
    head = plain_record(ctx, scene, cfg, args, flush, dist, world, local, args.workload, with_cpu=(world == 1))

    if rank == 0:
        line = {"metric": METRIC, "value": head["value"], "unit": "Mfrag/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": head["ms_per_step"], "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32+int64", "data": "synthetic (seeded)",
                "config": cfg}
        line.update({k: v for k, v in head.items() if k not in ("value", "unit", "ms_per_step")})
        other = "random" if args.workload == "terrain" else None
        if other and args.c0:
            c0_scene, c0_cfg = workload(other)
            sub = plain_record(ctx, c0_scene, c0_cfg, args, flush, None, 1, local, other, with_cpu=True)
            line["c0"] = dict(config=c0_cfg, **sub)
        if args.batch_frames > 0:
            line["batch"] = batched_section(ctx, args, flush)
        if args.diff_views > 0:
            line["differentiable"] = diff_section(ctx, args)
        if args.light_sprites > 0:
            line["deferred_light"] = light_section(ctx, args)
        line["summary"] = summary(line)
        print(json.dumps(line), flush=True)
    ctx.close()
    if dist:
        dist.destroy_process_group()


def summary(line):
    """The headline figures of every section in one short object, last on the line."""
    out = {f"{line['config']['workload'].split(',')[0]} frames/s": line["frames_per_s"],
           "e2e frames/s": line["e2e"]["frames_per_s"], "roofline frac (walked)": line["roofline"]["frac"],
           "frame roofline frac": line["frame_roofline"]["frac"],
           "cpu_baseline frames/s": line.get("cpu_baseline", {}).get("frames_per_s")}
    if "c0" in line:
        c0 = line["c0"]
        out.update({"c0 800x600 random 20k frames/s": c0["frames_per_s"], "c0 e2e frames/s": c0["e2e"]["frames_per_s"],
                    "c0 Mfrag/s": c0["value"], "c0 walked fragments/frame": c0["walked_fragments_per_frame"],
                    "c0 roofline frac (walked)": c0["roofline"]["frac"],
                    "c0 cpu_baseline frames/s": c0.get("cpu_baseline", {}).get("frames_per_s")})
    if "batch" in line:
        b = line["batch"]
        out.update({"batch batched frames/s": b["batched"]["frames_per_s"], "batch plain frames/s": b["plain"]["frames_per_s"],
                    "batch batched_over_plain": b["batched_over_plain"], "batch e2e frames/s": b["e2e"]["frames_per_s"]})
    if "differentiable" in line:
        df = line["differentiable"]
        out.update({"diff views/s atomic": df["atomic"]["views_per_s"],
                    "diff views/s deterministic": df["deterministic"]["views_per_s"],
                    "diff grad_rel_err_max": df["grad_rel_err_max"]})
    if "deferred_light" in line:
        dl = line["deferred_light"]
        out.update({"deferred light ms/frame (one call)": dl["ms_per_frame"],
                    "deferred light ms/frame (call per step)": dl["ms_per_frame_one_call_per_step"],
                    "deferred light parity": dl["parity_with_oracle"],
                    "deferred light cpu port frames/s": dl["cpu_oracle"]["frames_per_s"]})
    return out


if __name__ == "__main__":
    main()
