"""GPU parity of the alpha filter (Filter::Alpha) against the oracle.

An alpha-filtered model blends every visible fragment over the pixel in submission order,
source * (alpha / 255) + target * (1 - alpha / 255) packed with saturation after each fragment,
tests depth without writing it, and draws like a solid model when there is no colour target
(fillShape, fillerTemplates.h:387-441).  Prefilled colour and depth images make every blend
visible; frames mixing solid and alpha-filtered tasks check the runs' order; bit-exact.
"""
import dataclasses

import numpy as np
import pytest

from dfpsr_gb300 import scenes

pytestmark = pytest.mark.gpu


def _alpha_scene(seed, triangles=600, width=160, height=120, texture_size=32):
    s = scenes.random_triangles(seed=seed, triangles=triangles, width=width, height=height, texture_size=texture_size)
    return dataclasses.replace(s, filter=1)


def _prefilled(seed, h, w):
    rng = np.random.default_rng(seed)
    color = rng.integers(0, 2**32, size=(h, w), dtype=np.uint64).astype(np.uint32)
    depth = rng.uniform(0.0, 0.3, size=(h, w)).astype(np.float32)
    return color, depth


def _gpu(ctx, scene, color, depth, *, use_color=True, use_depth=True, pack_order=0, counting=True):
    import torch
    import dfpsr_gb300 as d
    h, w = scene.height, scene.width
    cov = torch.zeros((h, w), dtype=torch.int32, device="cuda") if counting else None
    ctx.set_counting(counting, cov)
    try:
        c, z = d.render_scene(ctx, scene, color, depth, use_color=use_color, use_depth=use_depth, pack_order=pack_order)
        stats = ctx.stats()
    finally:
        ctx.set_counting(False)
    return c, z, stats, (cov.cpu().numpy().view(np.uint32) if counting else None)


def _check(gpu, ref, label, counting=True):
    c, z, stats, cov = gpu
    rc, rz, info = ref
    if rc is not None:
        bad = np.argwhere(c != rc)
        assert len(bad) == 0, f"{label}: {len(bad)} colour pixels differ, first {bad[:4].tolist()}"
    if rz is not None:
        bad = np.argwhere(z.view(np.uint32) != rz.view(np.uint32))
        assert len(bad) == 0, f"{label}: {len(bad)} depth pixels differ, first {bad[:4].tolist()}"
    if counting:
        assert np.array_equal(cov, info["coverage"]), f"{label}: coverage differs"
        assert stats["fragments"] == info["fragments"], label


@pytest.mark.parametrize("pack_order", [0, 1, 2, 3])
def test_alpha_over_prefilled_colour_and_depth(ctx, pack_order):
    from oracle import port
    s = _alpha_scene(seed=40 + pack_order)
    color, depth = _prefilled(7 + pack_order, s.height, s.width)
    ref = port.render(s, color, depth, pack_order=pack_order, coverage=True)
    assert not np.array_equal(ref[0], color)  # the blends change the image
    assert np.array_equal(ref[1].view(np.uint32), depth.view(np.uint32))  # depth is only read
    for counting in (True, False):
        gpu = _gpu(ctx, s, color, depth, pack_order=pack_order, counting=counting)
        _check(gpu, ref, f"pack order {pack_order} counting {counting}", counting)


def test_alpha_without_depth_buffer(ctx):
    from oracle import port
    s = _alpha_scene(seed=50)
    color, _ = _prefilled(8, s.height, s.width)
    ref = port.render(s, color, None, use_depth=False, coverage=True)
    _check(_gpu(ctx, s, color, None, use_depth=False), ref, "no depth")


def test_alpha_without_colour_target_draws_depth_like_solid(ctx):
    from oracle import port
    s = _alpha_scene(seed=51)
    _, depth = _prefilled(9, s.height, s.width)
    ref = port.render(s, None, depth, use_color=False, coverage=True)
    solid = port.render(dataclasses.replace(s, filter=0), None, depth, use_color=False)
    assert np.array_equal(ref[1].view(np.uint32), solid[1].view(np.uint32))
    _check(_gpu(ctx, s, None, depth, use_color=False), ref, "depth only")


def test_alpha_dense_overlap(ctx):
    """400x300, 5000 overlapping random triangles: long per-tile lists, each pixel blending a few
    hundred fragments in order."""
    from oracle import port
    s = _alpha_scene(seed=52, triangles=5000, width=400, height=300, texture_size=64)
    color, depth = _prefilled(10, s.height, s.width)
    depth[:] = 0.0
    ref = port.render(s, color, depth, coverage=True)
    _check(_gpu(ctx, s, color, depth), ref, "dense")


def test_frame_mixing_solid_and_alpha_tasks(ctx):
    """renderer_begin, then solid, alpha, alpha, solid, alpha tasks, renderer_end: the frame runs as
    consecutive runs of each kind and must equal the models drawn one after another."""
    import torch
    import dfpsr_gb300 as d
    from oracle import port
    filters = (0, 1, 1, 0, 1)
    parts = [dataclasses.replace(scenes.random_triangles(seed=60 + k, triangles=300, width=160, height=128, texture_size=32),
                                 filter=f) for k, f in enumerate(filters)]
    color, depth = _prefilled(11, 128, 160)
    depth[:] = 0.0
    rc, rz = color.copy(), depth.copy()
    coverage = np.zeros((128, 160), np.uint32)
    fragments = 0
    for p in parts:
        rc, rz, info = port.render(p, rc, rz, coverage=True)
        coverage += info["coverage"]
        fragments += info["fragments"]
    models = [d.Model(ctx, p) for p in parts]
    cov = torch.zeros((128, 160), dtype=torch.int32, device="cuda")
    for repeat in range(3):  # the later frames go through the cached phase graphs where they repeat
        c, z = color.copy(), depth.copy()
        ctx.set_counting(True, cov)
        try:
            r = d.Renderer(ctx)
            r.begin(c, z)
            for m in models:
                r.give_task(m, m.camera)
            r.end()
            stats = ctx.stats()
        finally:
            ctx.set_counting(False)
        assert np.array_equal(c, rc), f"repeat {repeat}: {int((c != rc).sum())} colour pixels differ"
        assert np.array_equal(z.view(np.uint32), rz.view(np.uint32)), f"repeat {repeat}: depth differs"
        assert np.array_equal(cov.cpu().numpy().view(np.uint32), coverage), f"repeat {repeat}: coverage differs"
        assert stats["fragments"] == fragments
        r.destroy()
