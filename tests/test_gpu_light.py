"""GPU parity of the deferred light passes and draw_higher against the oracle (oracle/dsr_oracle.c,
itself pinned to the reference build): every byte and every float bit must be identical."""
import numpy as np
import pytest

from dfpsr_gb300 import scenes

pytestmark = pytest.mark.gpu

THREADS = 8  # the reference thread count whose row bands both sides use


def dev(a, dtype):
    import torch
    return torch.tensor(np.ascontiguousarray(a).view(dtype), device="cuda")


def host(t, dtype):
    return t.cpu().numpy().view(dtype)


def random_images(rng, h, w):
    normal = rng.integers(0, 2**32, size=(h, w), dtype=np.uint64).astype(np.uint32)
    light = rng.integers(0, 2**32, size=(h, w), dtype=np.uint64).astype(np.uint32) & np.uint32(0x7F7F7F7F)
    height = rng.uniform(-2, 2, size=(h, w)).astype(np.float32)
    return normal, light, height


def test_directed_light(ctx):
    import dfpsr_gb300 as d
    from oracle import port
    rng = np.random.default_rng(1)
    normal, light, _ = random_images(rng, 157, 203)
    for index, add in ((3, False), (5, True)):
        view, oview = d.ortho_view(-0.8, 64, index), port.ortho_view(-0.8, 64, index)
        want = port.directed_light(oview, light, normal, (0.3, -1.0, 0.2), 0.9, (255, 200, 100), add)
        got = dev(light, np.int32)
        ctx.light_directed(view, got, dev(normal, np.int32), (0.3, -1.0, 0.2), 0.9, (255, 200, 100), add)
        assert np.array_equal(host(got, np.uint32), want)


@pytest.mark.parametrize("shadows", [False, True])
def test_point_lights_with_row_bands(ctx, shadows):
    """Several lights in one pass against the oracle light after light; tall bounds exercise the
    reference's row bands, which restart its running sums."""
    import dfpsr_gb300 as d
    from oracle import port
    rng = np.random.default_rng(2)
    h, w = 600, 360
    normal, light, height = random_images(rng, h, w)
    view, oview = d.ortho_view(-0.8, 64, 2), port.ortho_view(-0.8, 64, 2)
    lights = []
    for _ in range(4):
        lights.append({"position": (rng.uniform(-2, 2), rng.uniform(0, 2), rng.uniform(-2, 2)), "radius": float(rng.uniform(2, 6)),
                       "intensity": float(rng.uniform(0.5, 1.5)), "color": tuple(int(c) for c in rng.integers(64, 256, 3))})
    cubes = [rng.uniform(0, 0.6, size=(6 * 64, 64)).astype(np.float32) for _ in lights] if shadows else [None] * 4
    want = light
    for l, cube in zip(lights, cubes):
        want = port.point_light(oview, (w // 2, h // 2), want, normal, height, l["position"], l["radius"], l["intensity"],
                                l["color"], cube, THREADS)
    assert (want != light).sum() > 20000
    got = dev(light, np.int32)
    gpu_lights = [dict(l, cube=dev(c, np.float32)) if c is not None else l for l, c in zip(lights, cubes)]
    ctx.light_points(view, (w // 2, h // 2), got, dev(normal, np.int32), dev(height, np.float32), gpu_lights, THREADS)
    assert np.array_equal(host(got, np.uint32), want)


def test_blend_light_every_pack_order(ctx):
    import torch
    from oracle import port
    rng = np.random.default_rng(3)
    diffuse, light, _ = random_images(rng, 97, 131)
    for order in range(4):
        target = torch.empty((97, 131), dtype=torch.int32, device="cuda")
        ctx.light_blend(target, dev(diffuse, np.int32), dev(light, np.int32), order)
        assert np.array_equal(host(target, np.uint32), port.blend_light(order, diffuse, light))


def test_draw_higher_many_sprites(ctx):
    """Overlapping sprites with transparent pixels, equal heights (the earliest wins), clipped
    placements and mixed pack orders, against the oracle's draw_higher sprite after sprite."""
    from oracle import port
    rng = np.random.default_rng(4)
    H, W = 120, 170
    th = rng.uniform(-1, 0.5, size=(H, W)).astype(np.float32)
    ta = rng.integers(0, 2**32, size=(H, W), dtype=np.uint64).astype(np.uint32)
    tb = rng.integers(0, 2**32, size=(H, W), dtype=np.uint64).astype(np.uint32)
    sprites, want = [], (th, ta, tb)
    for k in range(40):
        sh_, sw_ = int(rng.integers(8, 50)), int(rng.integers(8, 50))
        hgt = np.round(rng.uniform(-1, 1, size=(sh_, sw_)) * 4).astype(np.float32) / 4  # many equal heights
        hgt[rng.uniform(size=hgt.shape) < 0.15] = -np.inf
        a = rng.integers(0, 2**32, size=(sh_, sw_), dtype=np.uint64).astype(np.uint32)
        b = rng.integers(0, 2**32, size=(sh_, sw_), dtype=np.uint64).astype(np.uint32)
        left, top = int(rng.integers(-30, W)), int(rng.integers(-30, H))
        offset = float(np.float32(rng.choice([0.0, 0.25, -0.25])))
        ap, bp = int(rng.integers(0, 4)), int(rng.integers(0, 4))
        want = port.draw_higher((want[0], want[1], 1, want[2], 2), (hgt, a, ap, b, bp), left, top, offset)
        sprites.append({"height": dev(hgt, np.float32), "color_a": dev(a, np.int32), "color_b": dev(b, np.int32),
                        "left": left, "top": top, "offset": offset, "a_pack": ap, "b_pack": bp})
    gh, ga, gb = dev(th, np.float32), dev(ta, np.int32), dev(tb, np.int32)
    ctx.draw_higher(gh, ga, gb, sprites, a_pack=1, b_pack=2)
    assert np.array_equal(host(gh, np.uint32), want[0].view(np.uint32))
    assert np.array_equal(host(ga, np.uint32), want[1])
    assert np.array_equal(host(gb, np.uint32), want[2])


def test_deferred_light_pass_end_to_end(ctx):
    """Sprites, shadow cube maps from a depth-only batch, directed and point lights, blendLight."""
    import dfpsr_gb300 as d
    from dfpsr_gb300.sprite_pass import DeferredLightPass
    from oracle import light_pass
    m, _ = d.ortho_view(-0.7, 64, 0).arrays()
    scene = scenes.light_scene(seed=3, width=320, height=300, sprites=150, sprite_types=6, lights=4, radius_px=(60, 150),
                               caster_triangles=300, cube_resolution=64, light_space=(m[9:18], m[0:9]))
    out, light, height, diffuse, normal, cubes = light_pass.run(scene, THREADS)
    gpu = DeferredLightPass(ctx, scene, THREADS)
    got = gpu.run()
    assert np.array_equal(host(gpu.height, np.uint32), height.view(np.uint32))
    assert np.array_equal(host(gpu.diffuse, np.uint32), diffuse)
    assert np.array_equal(host(gpu.normal, np.uint32), normal)
    for k, cube in enumerate(cubes):
        assert np.array_equal(host(gpu.cubes[k], np.uint32), cube.view(np.uint32)), f"shadow cube {k}"
        assert (cube > 0).sum() > 100
    assert np.array_equal(host(gpu.light, np.uint32), light)
    assert np.array_equal(host(got, np.uint32), out)
    assert (out != 0).mean() > 0.3
    gpu.destroy()


def _pinned(a, pad=3):
    """A page-locked copy of a 2-D array of 4-byte pixels, with padded rows."""
    import torch
    h, w = a.shape
    dtype = torch.float32 if a.dtype == np.float32 else torch.int32
    buf = torch.zeros((h, w + pad), dtype=dtype).pin_memory().numpy()[:, :w]
    buf[:] = a.view(buf.dtype)
    return buf


@pytest.mark.parametrize("memory", ["pageable", "page-locked"])
def test_light_calls_and_draw_higher_take_host_images(ctx, memory):
    """The reference's light functions and draw_higher take host images: the same calls with
    pageable (staged) and page-locked (read and written in place) host images, shadow cubes and
    sprite sources give the oracle's results."""
    import dfpsr_gb300 as d
    from oracle import port
    place = (lambda a: np.ascontiguousarray(a).copy()) if memory == "pageable" else _pinned
    rng = np.random.default_rng(11)
    h, w = 300, 240
    normal, light, height = random_images(rng, h, w)
    view, oview = d.ortho_view(-0.8, 64, 1), port.ortho_view(-0.8, 64, 1)
    # directed light
    want = port.directed_light(oview, light, normal, (0.3, -1.0, 0.2), 0.9, (255, 200, 100), True)
    got = place(light)
    ctx.light_directed(view, got, place(normal), (0.3, -1.0, 0.2), 0.9, (255, 200, 100), True)
    assert np.array_equal(got.view(np.uint32), want)
    # point lights with shadow cubes
    lights = [{"position": (rng.uniform(-2, 2), rng.uniform(0, 2), rng.uniform(-2, 2)), "radius": float(rng.uniform(2, 6)),
               "intensity": float(rng.uniform(0.5, 1.5)), "color": tuple(int(c) for c in rng.integers(64, 256, 3))} for _ in range(3)]
    cubes = [rng.uniform(0, 0.6, size=(6 * 32, 32)).astype(np.float32) for _ in lights]
    want = light
    for l, cube in zip(lights, cubes):
        want = port.point_light(oview, (w // 2, h // 2), want, normal, height, l["position"], l["radius"], l["intensity"], l["color"],
                                cube, THREADS)
    got = place(light)
    host_cubes = [np.ascontiguousarray(c) if memory == "pageable" else _pinned(c, pad=0) for c in cubes]
    ctx.light_points(view, (w // 2, h // 2), got, place(normal), place(height),
                     [dict(l, cube=c) for l, c in zip(lights, host_cubes)], THREADS)
    assert np.array_equal(got.view(np.uint32), want)
    # blendLight
    target = place(np.zeros((h, w), np.uint32))
    ctx.light_blend(target, place(normal), place(light), 2)
    assert np.array_equal(target.view(np.uint32), port.blend_light(2, normal, light))
    # draw_higher with host sprites
    th = rng.uniform(-1, 0.5, size=(h, w)).astype(np.float32)
    ta = rng.integers(0, 2**32, size=(h, w), dtype=np.uint64).astype(np.uint32)
    tb = rng.integers(0, 2**32, size=(h, w), dtype=np.uint64).astype(np.uint32)
    sprites, expected = [], (th, ta, tb)
    for k in range(12):
        sh_, sw_ = int(rng.integers(8, 40)), int(rng.integers(8, 40))
        hgt = rng.uniform(-1, 1, size=(sh_, sw_)).astype(np.float32)
        a = rng.integers(0, 2**32, size=(sh_, sw_), dtype=np.uint64).astype(np.uint32)
        b = rng.integers(0, 2**32, size=(sh_, sw_), dtype=np.uint64).astype(np.uint32)
        left, top = int(rng.integers(-20, w)), int(rng.integers(-20, h))
        expected = port.draw_higher((expected[0], expected[1], 0, expected[2], 0), (hgt, a, 0, b, 0), left, top, 0.0)
        sprites.append({"height": place(hgt), "color_a": place(a), "color_b": place(b), "left": left, "top": top, "offset": 0.0,
                        "a_pack": 0, "b_pack": 0})
    gh, ga, gb = place(th), place(ta), place(tb)
    ctx.draw_higher(gh, ga, gb, sprites)
    assert np.array_equal(gh.view(np.uint32), expected[0].view(np.uint32))
    assert np.array_equal(ga.view(np.uint32), expected[1])
    assert np.array_equal(gb.view(np.uint32), expected[2])


@pytest.mark.parametrize("memory", ["device", "pageable", "page-locked"])
def test_sprite_frame_in_one_call(ctx, memory):
    """dsrg_sprite_frame (clears, draw_higher, directed light, the shadow batch, point lights and
    blendLight queued on the library's stream with two waits) gives the oracle's frame, with the
    frame images and sprite sources in device, pageable or page-locked memory, and equals the same
    frame made one call per step."""
    import dfpsr_gb300 as d
    from dfpsr_gb300.sprite_pass import BACKGROUND_HEIGHT, DeferredLightPass
    from oracle import light_pass
    m, _ = d.ortho_view(-0.7, 64, 2).arrays()
    scene = scenes.light_scene(seed=8, width=256, height=200, sprites=90, sprite_types=5, lights=3, radius_px=(50, 120),
                               caster_triangles=200, cube_resolution=32, light_space=(m[9:18], m[0:9]))
    out, light, height, diffuse, normal, cubes = light_pass.run(scene, THREADS)
    gpu = DeferredLightPass(ctx, scene, THREADS)
    steps_out = host(gpu.run_steps(), np.uint32).copy()
    assert np.array_equal(steps_out, out)
    if memory == "device":
        got = host(gpu.run(), np.uint32)
        assert np.array_equal(host(gpu.height, np.uint32), height.view(np.uint32))
        assert np.array_equal(host(gpu.light, np.uint32), light)
        assert np.array_equal(got, out)
    else:
        place = (lambda a: np.ascontiguousarray(a).copy()) if memory == "pageable" else _pinned
        H, W = scene.height, scene.width
        images = [place(np.full((H, W), 7.0, np.float32))] + [place(np.full((H, W), 0x01020304, np.uint32)) for _ in range(4)]
        sprites = d.SpriteArray([dict(s, height=place(host(s["height"], np.float32)), color_a=place(host(s["color_a"], np.uint32)),
                                      color_b=place(host(s["color_b"], np.uint32))) for s in _sprite_dicts(gpu)])
        ctx.sprite_frame(gpu.view, scene.center, images, (BACKGROUND_HEIGHT, 0, 0), sprites,
                         (scene.sun_direction, scene.sun_intensity, scene.sun_color), gpu.shadows, gpu.light_list, THREADS)
        assert np.array_equal(images[0].view(np.uint32), height.view(np.uint32))
        assert np.array_equal(images[1].view(np.uint32), diffuse)
        assert np.array_equal(images[2].view(np.uint32), normal)
        assert np.array_equal(images[3].view(np.uint32), light)
        assert np.array_equal(images[4].view(np.uint32), out)
    gpu.destroy()


def _sprite_dicts(gpu):
    out = []
    for i in range(gpu.sprites.count):
        s = gpu.sprites.array[i]
        h, a, b = gpu.sprites._keep[i]
        out.append({"height": h, "color_a": a, "color_b": b, "left": s.left, "top": s.top, "offset": s.offset})
    return out


def test_sprite_frame_first_call_on_a_fresh_context(built):
    """On a fresh context the large shadow triangles of 256 x 256 cube faces outgrow the row and
    tile-list buffers the shadow batch starts with; the batch is redone with grown buffers inside
    the call, and the first call already gives the oracle's frame (and so does the next one)."""
    import dfpsr_gb300 as d
    from dfpsr_gb300.sprite_pass import DeferredLightPass
    from oracle import light_pass
    m, _ = d.ortho_view(-0.7, 64, 1).arrays()
    scene = scenes.light_scene(seed=10, width=256, height=200, sprites=40, sprite_types=4, lights=2, radius_px=(60, 120),
                               caster_triangles=100, cube_resolution=256, light_space=(m[9:18], m[0:9]))
    out, *_ = light_pass.run(scene, THREADS)
    fresh = d.Context(0)
    try:
        gpu = DeferredLightPass(fresh, scene, THREADS)
        assert np.array_equal(host(gpu.run(), np.uint32), out)
        assert fresh.stats()["draw_records"] > 0  # the statistics of the checked shadow batch
        assert np.array_equal(host(gpu.run(), np.uint32), out)
        gpu.destroy()
    finally:
        fresh.close()


def test_sprite_frame_rejects_pageable_shadow_cubes(ctx):
    """Shadow cubes are read by the point lights after the shadow batch drew them: the frame takes
    them in device or page-locked memory only, and says so."""
    import dfpsr_gb300 as d
    from dfpsr_gb300.sprite_pass import BACKGROUND_HEIGHT, DeferredLightPass
    m, _ = d.ortho_view(-0.7, 64, 0).arrays()
    scene = scenes.light_scene(seed=9, width=64, height=64, sprites=4, sprite_types=2, lights=1, radius_px=(20, 30),
                               caster_triangles=20, cube_resolution=16, light_space=(m[9:18], m[0:9]))
    gpu = DeferredLightPass(ctx, scene, THREADS)
    pageable_cube = np.zeros((6 * 16, 16), np.float32)
    lights = [dict(l, cube=pageable_cube) for l in gpu.light_list]
    images = (gpu.height, gpu.diffuse, gpu.normal, gpu.light, gpu.output)
    with pytest.raises(d.DsrgError) as e:
        ctx.sprite_frame(gpu.view, scene.center, images, (BACKGROUND_HEIGHT, 0, 0), gpu.sprites,
                         (scene.sun_direction, scene.sun_intensity, scene.sun_color), None, lights, THREADS)
    assert e.value.status == 1 and "page-locked" in str(e.value)
    gpu.destroy()


def test_float_roots_equal_the_scalar_builds_double_roots(ctx):
    """The point lights take the scalar build's (float)sqrt((double)x) and (float)(1.0 / sqrt((double)x))
    as the correctly rounded float square root and reciprocal square root.  Checked on the device for
    every float of [1, 4), which covers every positive input (x -> 4x scales both sides by exactly 2,
    subnormal inputs included), and directly for zero and the subnormals, the largest floats up to
    infinity and the first NaNs, and negative inputs."""
    assert ctx.check_float_roots(0x3F800000, 1 << 24) == 0
    for first, count in ((0x00000000, 1 << 23), (0x7F000000, (1 << 23) + 2), (0x80000000, 1 << 16), (0xBF800000, 1 << 16)):
        assert ctx.check_float_roots(first, count) == 0, hex(first)


def test_benchmarked_light_pass_full_size(ctx):
    """The benchmarked deferred-light frame itself (scenes.light_scene(seed=2024): 1920x1080, 4096
    sprites, 16 shadowed point lights with 6 x 512 x 512 cube maps from a 2,000-triangle caster), as
    one dsrg_sprite_frame call, against the oracle's whole pass, image by image, bit for bit."""
    import os
    import dfpsr_gb300 as d
    from dfpsr_gb300.sprite_pass import DeferredLightPass
    from oracle import light_pass
    m, _ = d.ortho_view(-0.7, 64, 0).arrays()
    scene = scenes.light_scene(seed=2024, sprites=4096, light_space=(m[9:18], m[0:9]))
    workers = os.cpu_count() or 1
    out, light, height, diffuse, normal, cubes = light_pass.run(scene, THREADS, workers=workers)
    gpu = DeferredLightPass(ctx, scene, THREADS)
    got = host(gpu.run(), np.uint32)
    assert np.array_equal(host(gpu.height, np.uint32), height.view(np.uint32))
    assert np.array_equal(host(gpu.diffuse, np.uint32), diffuse)
    assert np.array_equal(host(gpu.normal, np.uint32), normal)
    for k, cube in enumerate(cubes):
        assert np.array_equal(host(gpu.cubes[k], np.uint32), cube.view(np.uint32)), f"shadow cube {k}"
    assert np.array_equal(host(gpu.light, np.uint32), light)
    assert np.array_equal(got, out)
    gpu.destroy()


def test_sprite_frame_without_sprites_lights_or_shadows(ctx):
    """A frame with no sprites, no point lights and no shadow batch: the clears, the directed light
    over the cleared normals and the blend, as the calls one by one make them."""
    import torch
    import dfpsr_gb300 as d
    H, W = 64, 96
    view = d.ortho_view(-0.7, 64, 3)
    images = [torch.zeros((H, W), dtype=torch.float32, device="cuda")] + \
             [torch.zeros((H, W), dtype=torch.int32, device="cuda") for _ in range(4)]
    sun = ((0.3, -1.0, 0.2), 0.8, (255, 220, 180))
    normal_word = 0x00C08040
    ctx.sprite_frame(view, (W // 2, H // 2), images, (-5.0, 0x11223344, normal_word), d.SpriteArray([]), sun, None, [], THREADS)
    assert (host(images[0], np.float32) == -5.0).all()
    assert (host(images[1], np.uint32) == 0x11223344).all()
    assert (host(images[2], np.uint32) == normal_word).all()
    normal = torch.full((H, W), normal_word, dtype=torch.int32, device="cuda")
    light = torch.zeros((H, W), dtype=torch.int32, device="cuda")
    ctx.light_directed(view, light, normal, sun[0], sun[1], sun[2], False)
    assert np.array_equal(host(images[3], np.uint32), host(light, np.uint32))
    out = torch.zeros((H, W), dtype=torch.int32, device="cuda")
    ctx.light_blend(out, images[1], light)
    assert np.array_equal(host(images[4], np.uint32), host(out, np.uint32))
    assert ctx.check_float_roots(0x3F800000, 0) == 0
