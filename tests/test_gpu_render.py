"""GPU parity of dsrg_model_render / dsrg_model_render_depth / dsrg_renderer_* against the oracle.

The bar is bit-exact: the oracle is pinned to the reference's exact (scalar, no-FMA)
build, and the GPU computes the same binary32 operations, so colour bytes, depth bits,
the per-pixel fragment counts and the fragment total must all be identical.
"""
import numpy as np
import pytest

from dfpsr_gb300 import scenes

pytestmark = pytest.mark.gpu


def gpu_render(ctx, scene, color=None, depth=None, *, use_color=True, use_depth=True, pack_order=0, counting=True):
    import torch
    import dfpsr_gb300 as d
    h, w = scene.height, scene.width
    cov = torch.zeros((h, w), dtype=torch.int32, device="cuda") if counting else None
    ctx.set_counting(counting, cov)
    c, dd = d.render_scene(ctx, scene, color, depth, use_color=use_color, use_depth=use_depth, pack_order=pack_order)
    stats = ctx.stats()
    ctx.set_counting(False)
    coverage = cov.cpu().numpy().view(np.uint32) if counting else None
    return c, dd, stats, coverage


def assert_same(scene, gpu, ref, label=""):
    from oracle import port  # noqa: F401
    c, d, stats, cov = gpu
    rc, rd, info = ref
    if rc is not None:
        diff = np.argwhere(c != rc)
        assert len(diff) == 0, f"{label}: {len(diff)} colour pixels differ, first {diff[:5].tolist()}"
    if rd is not None:
        diff = np.argwhere(d.view(np.uint32) != rd.view(np.uint32))
        assert len(diff) == 0, f"{label}: {len(diff)} depth pixels differ, first {diff[:5].tolist()}"
    if cov is not None and info.get("coverage") is not None:
        diff = np.argwhere(cov != info["coverage"])
        assert len(diff) == 0, f"{label}: coverage differs at {len(diff)} pixels, first {diff[:5].tolist()}"
    assert stats["fragments"] == info["fragments"], label


def run_case(ctx, scene, label, **kw):
    """Renders twice: counting fragments (every fragment is walked, coverage and total are
    compared) and not counting (the tile kernel's early depth culling is on); both must give
    the oracle's images."""
    from oracle import port
    gpu = gpu_render(ctx, scene, **kw)
    ref = port.render(scene, coverage=True, **{k: v for k, v in kw.items() if k in ("use_color", "use_depth", "pack_order")})
    assert_same(scene, gpu, ref, label)
    c, d, _, _ = gpu_render(ctx, scene, **dict(kw, counting=False))
    assert_same(scene, (c, d, {"fragments": ref[2]["fragments"]}, None), ref, label + " (culling)")
    return gpu


def test_random_triangles_small(ctx):
    run_case(ctx, scenes.random_triangles(seed=1234, triangles=300, width=160, height=120), "small")


def test_random_triangles_full_size(ctx):
    """800x600, 20k random triangles with a 256x256 mip-mapped texture."""
    c, d, stats, _ = run_case(ctx, scenes.random_triangles(seed=1234), "c0")
    assert stats["fragments"] > 100_000_000


def test_terrain_small(ctx):
    run_case(ctx, scenes.terrain(seed=3, grid=96, width=480, height=270, texture_size=128), "terrain")


def test_terrain_full_size(ctx):
    """1920x1080, 512x512 height grid (522k triangles), 1024x1024 mip-mapped texture."""
    run_case(ctx, scenes.terrain(seed=1234), "c1")


def test_near_plane_clipping(ctx):
    s = scenes.random_triangles(seed=9, triangles=3000, width=400, height=300)
    s.camera_location = scenes.camera_location((0.1, 0.2, -0.3), (0.0, 0.0, 1.0))
    run_case(ctx, s, "clipping")


def test_camera_inside_terrain(ctx):
    s = scenes.terrain(seed=5, grid=64, width=320, height=240, texture_size=64, camera_height=8.0, pitch_degrees=10.0)
    run_case(ctx, s, "low camera")


@pytest.mark.parametrize("variant", [
    dict(texture=False), dict(colors="white"), dict(colors="constant"), dict(light=True),
    dict(light=True, texture=False, colors="white"), dict(light=True, texture=False), dict(pyramid=False),
    dict(texture=False, colors="constant"), dict(light=True, colors="white"),
])
def test_shader_variants(ctx, variant):
    base = scenes.random_triangles(seed=11, triangles=1500, width=256, height=192)
    run_case(ctx, scenes.with_variant(base, **variant), str(variant))


@pytest.mark.parametrize("pack_order", [1, 2, 3])
def test_pack_orders(ctx, pack_order):
    run_case(ctx, scenes.random_triangles(seed=5, triangles=800, width=200, height=150), f"pack{pack_order}", pack_order=pack_order)


def test_prefilled_targets(ctx):
    """Drawing on existing colour and depth (the depth test reads the initial buffer)."""
    from oracle import port
    s = scenes.random_triangles(seed=21, triangles=1500, width=240, height=180)
    r = np.random.default_rng(2)
    color = r.integers(0, 2**32, (180, 240), dtype=np.uint64).astype(np.uint32)
    depth = r.uniform(0.0, 0.4, (180, 240)).astype(np.float32)
    gpu = gpu_render(ctx, s, color, depth)
    ref = port.render(s, color, depth, coverage=True)
    assert_same(s, gpu, ref, "prefilled")


def test_color_only_and_depth_only_targets(ctx):
    s = scenes.random_triangles(seed=22, triangles=1200, width=200, height=160)
    run_case(ctx, s, "color only", use_depth=False)
    run_case(ctx, s, "depth only", use_color=False)


def test_orthogonal_camera(ctx):
    s = scenes.random_triangles(seed=23, triangles=1500, width=256, height=200)
    s.perspective = False
    s.slope = 1.3
    run_case(ctx, s, "orthogonal")


def test_odd_width(ctx):
    run_case(ctx, scenes.random_triangles(seed=24, triangles=900, width=203, height=150), "odd width")


def test_model_render_depth(ctx):
    """model_renderDepth: 1x1 walk from each row's left edge (renderCore.cpp:343-443)."""
    import dfpsr_gb300 as d
    from oracle import port
    s = scenes.random_triangles(seed=25, triangles=2000, width=320, height=240)
    m = d.Model(ctx, s)
    depth = np.zeros((240, 320), np.float32)
    ctx.set_counting(True)
    ctx.render_depth(m, m.camera, depth)
    stats = ctx.stats()
    ctx.set_counting(False)
    ref, info = port.render_depth(s)
    assert np.array_equal(depth.view(np.uint32), ref.view(np.uint32))
    assert stats["fragments"] == info["fragments"]
    culled = np.zeros((240, 320), np.float32)  # not counting: early depth culling on
    ctx.render_depth(m, m.camera, culled)
    assert np.array_equal(culled.view(np.uint32), ref.view(np.uint32))


def test_renderer_tasks_equal_sequential_model_renders(ctx):
    """renderer_begin + several giveTask + renderer_end equals model_render of the tasks in order."""
    import dfpsr_gb300 as d
    from oracle import port
    a = scenes.random_triangles(seed=31, triangles=700, width=256, height=192)
    b = scenes.random_triangles(seed=32, triangles=700, width=256, height=192)
    b.model_to_world = np.array([0.3, -0.2, 0.5, 1, 0, 0, 0, 1, 0, 0, 0, 1], np.float32)
    ma, mb = d.Model(ctx, a), d.Model(ctx, b)
    color = np.zeros((192, 256), np.uint32)
    depth = np.zeros((192, 256), np.float32)
    r = ctx.renderer()
    r.begin(color, depth)
    assert r.takes_triangles
    r.give_task(ma)
    r.give_task(mb)
    r.end()
    assert not r.takes_triangles
    rc, rd, _ = port.render(a)
    rc, rd, _ = port.render(b, rc, rd)
    assert np.array_equal(color, rc)
    assert np.array_equal(depth.view(np.uint32), rd.view(np.uint32))


def test_renderer_call_order_errors(ctx):
    import dfpsr_gb300 as d
    r = ctx.renderer()
    with pytest.raises(d.DsrgError, match="renderer_end without renderer_begin"):
        r.end()
    color = np.zeros((16, 16), np.uint32)
    r.begin(color)
    with pytest.raises(d.DsrgError, match="renderer_begin on the same renderer twice"):
        r.begin(color)
    r.end()


def test_device_resident_targets(ctx):
    """Images already in HBM (onDevice) give the same result as host images."""
    import torch
    import dfpsr_gb300 as d
    from oracle import port
    s = scenes.random_triangles(seed=41, triangles=1500, width=320, height=240)
    m = d.Model(ctx, s)
    color = torch.zeros((240, 320), dtype=torch.int32, device="cuda")
    depth = torch.zeros((240, 320), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    ctx.render(m, m.camera, color, depth)
    rc, rd, _ = port.render(s)
    assert np.array_equal(color.cpu().numpy().view(np.uint32), rc)
    assert np.array_equal(depth.cpu().numpy().view(np.uint32), rd.view(np.uint32))


def test_page_locked_host_targets(ctx):
    """Page-locked host images (drawn in place through their device addresses, no staging copies),
    with padded rows and prefilled contents, in a frame of solid and alpha-filtered tasks with the
    wireframe overlay (every pass that reads or writes the targets): identical to the oracle."""
    import dataclasses
    import torch
    import dfpsr_gb300 as d
    from oracle import port
    h, w = 150, 230
    base = scenes.random_triangles(seed=43, triangles=900, width=w, height=h, texture_size=32)
    parts = [base, dataclasses.replace(scenes.random_triangles(seed=44, triangles=500, width=w, height=h, texture_size=32),
                                       filter=1)]
    rng = np.random.default_rng(45)
    color0 = rng.integers(0, 2**32, size=(h, w), dtype=np.uint64).astype(np.uint32)
    depth0 = rng.uniform(0.0, 0.2, size=(h, w)).astype(np.float32)
    o = port.OracleRenderer()
    rc, rz = color0.copy(), depth0.copy()
    o.begin(rc, rz)
    pms = [port.PreparedModel(p) for p in parts]
    for pm, p in zip(pms, parts):
        o.give_task(pm, p.model_to_world, pm.cam)
    rc, rz, _ = o.end(debug_wireframe=True)
    c = torch.zeros((h, w + 7), dtype=torch.int32).pin_memory().numpy()[:, :w].view(np.uint32)
    z = torch.zeros((h, w + 1), dtype=torch.float32).pin_memory().numpy()[:, :w]
    models = [d.Model(ctx, p) for p in parts]
    r = d.Renderer(ctx)
    for _ in range(2):
        c[:], z[:] = color0, depth0
        r.begin(c, z)
        for m, p in zip(models, parts):
            r.give_task(m, m.camera, p.model_to_world)
        r.end(debug_wireframe=True)
        assert np.array_equal(c, rc), f"{int((c != rc).sum())} colour pixels differ"
        assert np.array_equal(z.view(np.uint32), rz.view(np.uint32))
    r.destroy()


def test_texture_pyramid_matches_oracle(ctx):
    import dfpsr_gb300 as d
    from oracle import port
    r = np.random.default_rng(3)
    for (w, h, levels) in [(256, 256, 16), (64, 16, 3), (32, 128, 16), (8, 8, 1)]:
        pixels = r.integers(0, 2**32, (h, w), dtype=np.uint64).astype(np.uint32)
        fields, pyramid = d.Texture(ctx, pixels, levels).read()
        ot = port.OracleTexture(pixels, levels)
        assert list(fields) == ot.t.fields()
        assert np.array_equal(pyramid, ot.t.array())
