"""GPU texture creation (dsrg_texture_create / dsrg_texture_create_many) against the oracle, which the
CPU tests pin to the reference: the linear resize to the next powers of two (every path of
filter_resize: copy, vertical only, horizontal only, both, and the two-step upscale) and the
integer pyramid, from host and device images, one at a time and many per call; bit-exact."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SIZES = [(1, 1, 16), (3, 5, 16), (5, 3, 16), (17, 16, 16), (16, 17, 16), (20, 12, 16), (12, 20, 3), (100, 60, 16),
         (60, 100, 2), (64, 48, 16), (48, 64, 16), (255, 257, 16), (129, 31, 5), (1000, 600, 16), (33, 2, 16),
         (256, 256, 16), (512, 128, 4), (8, 8, 1)]


def _image(w, h, seed):
    return np.random.default_rng(seed).integers(0, 2**32, size=(h, w), dtype=np.uint64).astype(np.uint32)


def _same(tex, pixels, levels):
    from oracle import port
    fields, pyramid = tex.read()
    ot = port.OracleTexture(pixels, levels)
    assert list(fields) == ot.t.fields(), (pixels.shape, levels)
    assert np.array_equal(pyramid, ot.t.array()), (pixels.shape, levels)


def test_texture_create_any_size_matches_oracle(ctx):
    import dfpsr_gb300 as d
    for i, (w, h, levels) in enumerate(SIZES):
        pixels = _image(w, h, i)
        _same(d.Texture(ctx, pixels, levels), pixels, levels)


def test_texture_create_many_host_and_device(ctx):
    """One call for every size: host images, device images and strided device views mixed."""
    import torch
    import dfpsr_gb300 as d
    images, sources, levels = [], [], []
    for i, (w, h, lv) in enumerate(SIZES):
        pixels = _image(w, h, 100 + i)
        images.append(pixels)
        levels.append(lv)
        if i % 3 == 0:
            sources.append(pixels)
        elif i % 3 == 1:
            sources.append(torch.from_numpy(pixels.view(np.int32)).cuda())
        else:  # a view into a wider tensor: rows further apart than the image is wide
            wide = torch.zeros((h, w + 7), dtype=torch.int32, device="cuda")
            wide[:, 3:3 + w] = torch.from_numpy(pixels.view(np.int32)).cuda()
            sources.append(wide[:, 3:3 + w])
    textures = d.Texture.create_many(ctx, sources, levels)
    assert len(textures) == len(SIZES)
    for tex, pixels, lv in zip(textures, images, levels):
        _same(tex, pixels, lv)


def test_model_with_a_texture_of_any_size_renders_like_the_oracle(ctx):
    """A model whose texture is not a power of two renders exactly like the oracle's."""
    import dataclasses
    import dfpsr_gb300 as d
    from dfpsr_gb300 import scenes
    from oracle import port
    s = scenes.random_triangles(seed=71, triangles=400, width=160, height=120, texture_size=0)
    s = dataclasses.replace(s, diffuse=_image(90, 70, 7), diffuse_levels=16)
    c, z = d.render_scene(ctx, s)
    rc, rz, _ = port.render(s)
    assert np.array_equal(c, rc) and np.array_equal(z.view(np.uint32), rz.view(np.uint32))


def test_texture_create_errors(ctx):
    import dfpsr_gb300 as d
    with pytest.raises(d.DsrgError):
        d.Texture(ctx, np.zeros((4, 4), np.uint32), 0)
    with pytest.raises(d.DsrgError):
        d.Texture(ctx, np.zeros((4, 40000), np.uint32), 1)
    img = d.image_struct(np.zeros((4, 4), np.uint32), 7)  # no such pack order
    import ctypes as C
    out = (C.c_void_p * 1)()
    r = np.array([1], np.int32)
    assert ctx._l.dsrg_texture_create_many(ctx.handle, 1, (d.Image * 1)(img), r.ctypes.data, out) == 1
    assert out[0] is None


def test_texture_create_from_every_pack_order(ctx):
    """Images in BGRA, ARGB and ABGR order (and RGBA) through every resize path: the GPU texture
    equals the oracle's, which the CPU tests pin to the reference's texture_create_RgbaU8."""
    import dfpsr_gb300 as d
    from oracle import port
    sizes = [(16, 16, 16), (16, 10, 16), (16, 20, 4), (10, 16, 16), (20, 16, 16), (12, 20, 3), (100, 60, 16), (33, 2, 16)]
    images, orders, levels = [], [], []
    for i, (w, h, lv) in enumerate(sizes):
        for order in range(4):
            images.append(_image(w, h, 300 + 4 * i + order))
            orders.append(order)
            levels.append(lv)
    textures = d.Texture.create_many(ctx, images, levels, pack_orders=orders)
    for tex, pixels, order, lv in zip(textures, images, orders, levels):
        fields, pyramid = tex.read()
        ot = port.OracleTexture(pixels, lv, pack_order=order)
        assert list(fields) == ot.t.fields(), (pixels.shape, order)
        assert np.array_equal(pyramid, ot.t.array()), (pixels.shape, order)
