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
