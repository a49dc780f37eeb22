"""dsrg_model_render_depth_noalloc: depth rendering for callers that must not allocate GPU memory
during a call (for example a frame loop held to a no-allocation rule after start-up, since
cudaMalloc and cudaFree synchronise the whole device).

The entry point is called through the C ABI and must produce exactly what the allocating
dsrg_model_render_depth produces, on two calls in a row (the shared scratch array keeps the
previous call's contents, so the second call checks that nothing stale leaks through).
This file is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

from dfpsr_gb300 import scenes

pytestmark = pytest.mark.gpu


def _noalloc(ctx, model, depth):
    import dfpsr_gb300 as d
    t = np.ascontiguousarray(model.transform, np.float32)
    img = d.image_struct(depth)
    return d.lib().dsrg_model_render_depth_noalloc(ctx.handle, model.handle, t.ctypes.data, C.byref(model.camera), C.byref(img))


def test_no_alloc_depth_matches_allocating_entry_point(ctx):
    import torch
    import dfpsr_gb300 as d
    first = scenes.random_triangles(seed=51, triangles=1500, width=512, height=512)
    second = scenes.random_triangles(seed=52, triangles=900, width=384, height=256)
    second.camera_location = scenes.camera_location((0.3, -0.2, -2.5), (-0.1, 0.05, 1.0))
    for scene in (first, second):
        model = d.Model(ctx, scene)
        base = torch.rand((scene.height, scene.width), device="cuda") * 0.2
        expected = base.clone()
        got = base.clone()
        torch.cuda.synchronize()
        ctx.render_depth(model, model.camera, expected)
        status = _noalloc(ctx, model, got)
        assert status == 0, d.lib().dsrg_context_last_error(ctx.handle)
        torch.cuda.synchronize()
        assert torch.equal(got.view(torch.int32), expected.view(torch.int32))
        assert int((got != base).sum()) > 1000  # the call drew something


def test_no_alloc_rejects_host_images_and_oversized_targets(ctx):
    import torch
    import dfpsr_gb300 as d
    scene = scenes.random_triangles(seed=53, triangles=50, width=64, height=64)
    model = d.Model(ctx, scene)
    host = np.zeros((64, 64), np.float32)
    assert _noalloc(ctx, model, host) == 1
    assert b"device memory" in d.lib().dsrg_context_last_error(ctx.handle)
    big = torch.zeros((1025, 64), device="cuda")
    assert _noalloc(ctx, model, big) == 5
    assert b"DSRG_NOALLOC_MAX_SIDE" in d.lib().dsrg_context_last_error(ctx.handle)


def test_no_alloc_takes_no_device_memory_after_a_warm_up_call(ctx):
    """The property the entry point exists for: once a first call has loaded its device code,
    further calls leave the device's free memory as it was."""
    import torch
    import dfpsr_gb300 as d
    scene = scenes.random_triangles(seed=54, triangles=2000, width=640, height=480)
    model = d.Model(ctx, scene)
    depth = torch.zeros((480, 640), device="cuda")
    torch.cuda.synchronize()
    assert _noalloc(ctx, model, depth) == 0  # warm-up
    torch.cuda.synchronize()
    free_before, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        depth.zero_()
        assert _noalloc(ctx, model, depth) == 0, d.lib().dsrg_context_last_error(ctx.handle)
    torch.cuda.synchronize()
    free_after, _ = torch.cuda.mem_get_info()
    assert free_after == free_before


def test_no_alloc_rejects_views_beyond_its_tile_list_limit(ctx):
    """Screen-filling triangles at 1024 x 1024 need more (tile, triangle) pairs than
    DSRG_NOALLOC_MAX_BIN_ENTRIES: the call is refused before it draws, leaving the image as it was."""
    import torch
    import dfpsr_gb300 as d
    pairs = 700
    scene = scenes.random_triangles(seed=55, triangles=2 * pairs, width=1024, height=1024)
    # each pair: one triangle wider than the view at a depth of its own, in both windings (one of
    # the two faces the camera): about 700 drawn triangles over all 4,096 tiles, 700k pixel rows
    z = np.repeat(np.linspace(-1.0, 1.0, pairs, dtype=np.float32), 2)
    corners = np.array([[-3.0, -3.0], [3.0, -3.0], [0.0, 3.0]], np.float32)
    positions = np.zeros((2 * pairs, 3, 3), np.float32)
    positions[:, :, :2] = corners
    positions[1::2] = positions[1::2, ::-1]
    positions[:, :, 2] = z[:, None]
    scene.positions = positions.reshape(-1, 3)
    model = d.Model(ctx, scene)
    depth = torch.rand((1024, 1024), device="cuda") * 0.01
    before = depth.clone()
    torch.cuda.synchronize()
    assert _noalloc(ctx, model, depth) == 5
    assert b"DSRG_NOALLOC_MAX_BIN_ENTRIES" in d.lib().dsrg_context_last_error(ctx.handle)
    torch.cuda.synchronize()
    assert torch.equal(depth.view(torch.int32), before.view(torch.int32))
