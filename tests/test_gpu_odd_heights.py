"""GPU parity on targets of odd height, against the oracle, bit for bit.

On the last row of an odd-height target the reference's row pair has no lower row: the filler
empties that row's interval but bounds its run of full quads with the row as it was, and points
the lower row's pixels at the upper row (fillerTemplates.h:285-306).  Along that run a triangle
therefore tests its lower lanes against the upper row's depth and writes them after its upper
lanes, so the row keeps the last lane that passed, not the nearest fragment.  The tile pass leaves
that row of depth-tested frames to an ordered pass (odd_row_kernel); without a depth buffer the
last triangle wins with its lower lane's colour; the alpha filter blends the lower lane over the
colour both lanes read.  Every resolve mode, prefilled targets, orthographic cameras, colour-only
and depth-only targets, the renderer, the batch and windows of more records than one pass of the
ordered kernel holds are covered.
"""
import dataclasses

import numpy as np
import pytest

from dfpsr_gb300 import scenes
from test_gpu_render import assert_same, gpu_render, run_case

pytestmark = pytest.mark.gpu


def _scene(w, h, n, seed, texture_size=32, **kw):
    s = scenes.random_triangles(seed=seed, triangles=n, width=w, height=h, texture_size=texture_size)
    if kw.get("ortho"):
        s.perspective = False
        s.slope = 1.3
    if kw.get("alpha"):
        s = dataclasses.replace(s, filter=1)
    return s


@pytest.fixture
def tuned(ctx):
    """Restores the context's tuning after a test that changes it."""
    saved = ctx.tuning()
    yield ctx
    ctx.set_tuning(threads_per_tile=saved["threads_per_tile"], ctas_per_sm=saved["ctas_per_sm"],
                   small_rows=saved["small_rows"], small_width=saved["small_width"], graphs=bool(saved["graphs"]),
                   resolve=saved["resolve"])


@pytest.mark.parametrize("w,h,n", [(1, 57, 300), (64, 1, 300), (97, 3, 400), (199, 151, 2000), (301, 33, 2500)])
@pytest.mark.parametrize("resolve", [0, 1, 2])
def test_odd_heights_every_resolve_mode(tuned, w, h, n, resolve):
    tuned.set_tuning(resolve=resolve)
    run_case(tuned, _scene(w, h, n, seed=w * 7 + h), f"{w}x{h} resolve {resolve}")


def test_random_triangles_800x601(ctx):
    """The 800x600 random-triangle configuration (20k triangles, 256x256 mip-mapped texture) one row taller."""
    c, d, stats, _ = run_case(ctx, scenes.random_triangles(seed=1234, width=800, height=601), "800x601")
    assert stats["fragments"] > 100_000_000


def test_terrain_odd_height(ctx):
    run_case(ctx, scenes.terrain(seed=3, grid=96, width=481, height=271, texture_size=128), "terrain 481x271")


def test_odd_height_orthogonal_and_pack_orders(ctx):
    run_case(ctx, _scene(199, 151, 2000, seed=12, ortho=True), "orthogonal")
    for pack_order in (1, 2, 3):
        run_case(ctx, _scene(123, 45, 900, seed=30 + pack_order), f"pack {pack_order}", pack_order=pack_order)


def test_odd_height_colour_only_and_depth_only(ctx):
    s = _scene(203, 77, 1500, seed=22)
    run_case(ctx, s, "colour only", use_depth=False)
    run_case(ctx, s, "depth only", use_color=False)


def test_odd_height_prefilled_targets(ctx):
    from oracle import port
    s = _scene(240, 181, 1500, seed=21)
    r = np.random.default_rng(2)
    color = r.integers(0, 2**32, (181, 240), dtype=np.uint64).astype(np.uint32)
    depth = r.uniform(0.0, 0.4, (181, 240)).astype(np.float32)
    gpu = gpu_render(ctx, s, color, depth)
    assert_same(s, gpu, port.render(s, color, depth, coverage=True), "prefilled")
    culled = gpu_render(ctx, s, color, depth, counting=False)
    rc, rd, info = port.render(s, color, depth)
    assert_same(s, (culled[0], culled[1], {"fragments": info["fragments"]}, None), (rc, rd, info), "prefilled (culling)")


def test_odd_height_many_records_per_bottom_tile(ctx):
    """3000 large triangles over a 48x33 target: each bottom tile's last row is reached by more
    records than one window of the ordered pass holds, so the windows are split by record index."""
    run_case(ctx, _scene(48, 33, 3000, seed=14), "48x33 dense")
    run_case(ctx, _scene(48, 33, 3000, seed=15, ortho=True), "48x33 dense orthogonal")


@pytest.mark.parametrize("use_depth", [True, False])
def test_odd_height_alpha_filter(ctx, use_depth):
    from oracle import port
    s = _scene(199, 151, 1500, seed=13, alpha=True)
    r = np.random.default_rng(5)
    color = r.integers(0, 2**32, (151, 199), dtype=np.uint64).astype(np.uint32)
    depth = r.uniform(0.0, 0.3, (151, 199)).astype(np.float32) if use_depth else None
    gpu = gpu_render(ctx, s, color, depth, use_depth=use_depth)
    ref = port.render(s, color, depth, use_depth=use_depth, coverage=True)
    assert_same(s, gpu, ref, f"alpha depth={use_depth}")


def test_odd_height_renderer_with_solid_and_alpha_tasks(ctx):
    """renderer_begin, a solid task, an alpha-filtered task and another solid task, renderer_end."""
    import dfpsr_gb300 as d
    from oracle import port
    h, w = 143, 211
    parts = [_scene(w, h, 900, seed=61), _scene(w, h, 600, seed=62, alpha=True), _scene(w, h, 900, seed=63)]
    parts[2].model_to_world = np.array([0.2, -0.1, 0.3, 1, 0, 0, 0, 1, 0, 0, 0, 1], np.float32)
    o = port.OracleRenderer()
    rc, rz = np.zeros((h, w), np.uint32), np.zeros((h, w), np.float32)
    o.begin(rc, rz)
    pms = [port.PreparedModel(p) for p in parts]
    for pm, p in zip(pms, parts):
        o.give_task(pm, p.model_to_world, pm.cam)
    rc, rz, _ = o.end()
    models = [d.Model(ctx, p) for p in parts]
    color, depth = np.zeros((h, w), np.uint32), np.zeros((h, w), np.float32)
    r = ctx.renderer()
    r.begin(color, depth)
    for m, p in zip(models, parts):
        r.give_task(m, m.camera, p.model_to_world)
    r.end()
    assert np.array_equal(color, rc), f"{int((color != rc).sum())} colour pixels differ"
    assert np.array_equal(depth.view(np.uint32), rz.view(np.uint32))


def test_odd_height_frames_in_a_batch(ctx):
    """Frames of odd and even heights, with and without depth buffers, in one batch."""
    import dfpsr_gb300 as d
    from oracle import port
    specs = [(65, 33, 800, True), (64, 64, 800, True), (129, 97, 1500, True), (33, 17, 400, False), (200, 151, 2500, True)]
    frames = []
    b = ctx.batch()
    for i, (w, h, n, use_depth) in enumerate(specs):
        s = _scene(w, h, n, seed=70 + i)
        m = d.Model(ctx, s)
        color = np.zeros((h, w), np.uint32)
        depth = np.zeros((h, w), np.float32) if use_depth else None
        f = b.add_frame(color, depth)
        b.give_task(f, m, m.camera)
        frames.append((s, m, color, depth, use_depth))
    b.render()
    for s, m, color, depth, use_depth in frames:
        rc, rd, _ = port.render(s, use_depth=use_depth)
        assert np.array_equal(color, rc), f"{s.width}x{s.height}: {int((color != rc).sum())} colour pixels differ"
        if use_depth:
            assert np.array_equal(depth.view(np.uint32), rd.view(np.uint32)), f"{s.width}x{s.height} depth"
    b.destroy()
