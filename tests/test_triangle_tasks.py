"""renderer_giveTask_triangle (pre-projected triangles with their own colours, texture coordinates,
textures, filter and camera) mixed with model tasks in one frame: the oracle against the reference
(CPU, where the reference was built here) and the GPU against the oracle, bit-exact.  Some
triangles cross the near plane (the clipping path works from the given camera-space corners)."""
import dataclasses

import numpy as np
import pytest

from dfpsr_gb300 import scenes


def _inputs(seed=5, width=240, height=180):
    rng = np.random.default_rng(seed)
    a = scenes.random_triangles(seed=seed, triangles=300, width=width, height=height, texture_size=32)
    b = dataclasses.replace(scenes.random_triangles(seed=seed + 1, triangles=200, width=width, height=height, texture_size=32),
                            filter=1)

    def triangles(n, near):
        centers = np.stack([rng.uniform(-1.2, 1.2, n), rng.uniform(-1.0, 1.0, n), rng.uniform(-1.0, 1.5, n)], axis=1)
        if near:
            centers[: n // 5, 2] = rng.uniform(-3.4, -2.6, n // 5)  # around the camera at z = -3: clipped
        world = centers[:, None, :] + rng.uniform(-0.5, 0.5, size=(n, 3, 3))
        colors = rng.integers(0, 256, size=(n, 3, 4)).astype(np.float32) / np.float32(255.0)
        tex = rng.uniform(0.0, 1.0, size=(n, 3, 4)).astype(np.float32)
        return world.astype(np.float32), colors, tex

    t1 = triangles(150, True)
    t2 = triangles(80, False)
    texture = scenes.noise_texture(rng, 32)
    color = rng.integers(0, 2**32, size=(height, width), dtype=np.uint64).astype(np.uint32)
    return a, b, t1, t2, texture, color


def _project(cam, world):
    from oracle import port
    cs, is_, flat = port.world_to_screen(cam, world.reshape(-1, 3))
    n = world.shape[0]
    return cs.reshape(n, 3, 3), is_.reshape(n, 3, 2), flat.reshape(n, 3, 2)


def _oracle(inputs):
    from oracle import port
    a, b, t1, t2, texture, color = inputs
    cam = port.camera_desc(a)
    r = port.OracleRenderer()
    r.begin(color, np.zeros(color.shape, np.float32))
    pa, pb = port.PreparedModel(a), port.PreparedModel(b)
    tex = port.OracleTexture(texture, 16)
    r.give_task(pa, a.model_to_world, cam)
    r.give_triangles(*_project(cam, t1[0]), t1[1], t1[2], tex, None, 0, cam)
    r.give_task(pb, b.model_to_world, cam)
    r.give_triangles(*_project(cam, t2[0]), t2[1], t2[2], None, None, 1, cam)
    c, z, info = r.end()
    return c, z, info["fragments"]


def test_oracle_triangle_tasks_equal_reference(built):
    from oracle import port, ref
    if not ref.available("exact"):
        pytest.skip("the reference was not built from source on this machine")
    inputs = _inputs()
    a, b, t1, t2, texture, color = inputs
    cam = port.camera_desc(a)
    rr = ref.RefRenderer()
    rr.begin(color, np.zeros(color.shape, np.float32))
    ma, mb = ref.RefModel(a), ref.RefModel(b)
    tex = ref.RefTexture(ma.lib, texture, 16)
    rr.give_task(ma, a.model_to_world, cam)
    rr.give_triangles(*_project(cam, t1[0]), t1[1], t1[2], tex, None, 0, cam)
    rr.give_task(mb, b.model_to_world, cam)
    rr.give_triangles(*_project(cam, t2[0]), t2[1], t2[2], None, None, 1, cam)
    rc, rz = rr.end()
    oc, oz, _ = _oracle(inputs)
    assert np.array_equal(oc, rc), f"{int((oc != rc).sum())} colour pixels differ"
    assert np.array_equal(oz.view(np.uint32), rz.view(np.uint32))
    assert not np.array_equal(oc, color)


@pytest.mark.gpu
def test_gpu_triangle_tasks_match_oracle(ctx):
    import dfpsr_gb300 as d
    from oracle import port
    inputs = _inputs()
    a, b, t1, t2, texture, color = inputs
    oc, oz, fragments = _oracle(inputs)
    cam = d.camera_struct(a)
    pcam = port.camera_desc(a)

    def corners(world):
        cs, is_, flat = _project(pcam, world)
        out = np.zeros(world.shape[:2], d.PROJECTED_POINT)
        out["cs"], out["is"], out["flat"] = cs, is_, flat
        return out

    # the host projection helper equals the oracle's
    got = d.world_to_screen(cam, t1[0])
    assert np.array_equal(got.view(np.uint8), corners(t1[0]).view(np.uint8))
    r = d.Renderer(ctx)
    c, z = color.copy(), np.zeros(color.shape, np.float32)
    ctx.set_counting(True, None)
    try:
        r.begin(c, z)
        ci, _ = r.images()
        assert ci.width == color.shape[1] and ci.data is not None
        ma, mb = d.Model(ctx, a), d.Model(ctx, b)
        tex = d.Texture(ctx, texture, 16)
        r.give_task(ma, cam, a.model_to_world)
        r.give_triangles(corners(t1[0]), t1[1], t1[2], tex, None, 0, cam)
        r.give_task(mb, cam, b.model_to_world)
        r.give_triangles(corners(t2[0]), t2[1], t2[2], None, None, 1, cam)
        r.end()
        stats = ctx.stats()
    finally:
        ctx.set_counting(False)
    ci, zi = r.images()
    assert ci.data is None and zi.data is None  # only while the renderer takes triangles
    assert np.array_equal(c, oc), f"{int((c != oc).sum())} colour pixels differ"
    assert np.array_equal(z.view(np.uint32), oz.view(np.uint32))
    assert stats["fragments"] == fragments
    with pytest.raises(d.DsrgError) as e:
        r.give_triangles(corners(t2[0][:1]), t2[1][:1], t2[2][:1], None, None, 0, cam)
    assert e.value.status == 4
    r.destroy()
