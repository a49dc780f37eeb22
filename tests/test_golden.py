"""Parity pinned to the reference's own known answers and outputs (tests/golden/).

texture_kats.json holds the assertions of Source/test/tests/TextureTest.cpp; render_*.npz
hold seeded scenes with the images the reference itself (exact build) rendered for them.
The oracle must reproduce both on any machine; the GPU must reproduce the renders.
"""
import glob
import json
import os

import numpy as np
import pytest

from conftest import ROOT

GOLDEN = os.path.join(ROOT, "tests", "golden")


def kats():
    with open(os.path.join(GOLDEN, "texture_kats.json")) as f:
        return json.load(f)


FIELD_ORDER = ["log2width", "log2height", "maxMipLevel", "startOffset", "maxLevelMask",
               "minWidthOrMask", "minHeightOrMask", "maxWidthAndMask", "maxHeightAndMask"]


def test_oracle_texture_known_answers(built):
    import ctypes as C
    from oracle import port
    data = kats()
    checked = 0
    for block in data["textures"]:
        tex = port.OracleTexture(empty=(block["log2w"], block["log2h"], block["maxMip"]))
        t = tex.ref()
        l = port.lib()
        fields = dict(zip(FIELD_ORDER, tex.t.fields()))
        for name, value in block["fields"].items():
            if name == "MaxWidth":
                assert 1 << fields["log2width"] == value
            elif name == "MaxHeight":
                assert 1 << fields["log2height"] == value
            elif name == "SmallestMipLevel":
                assert fields["maxMipLevel"] == value
            elif name == "hasPyramid":
                assert (fields["maxMipLevel"] != 0) == bool(value)
            else:
                assert fields[name] == value, name
            checked += 1
        for mip, expected in block["layer"]:
            assert l.or_texture_pixel_offset_to_layer(t, mip) == expected
            checked += 1
        for x, y, mip, expected in block["offset"]:
            assert l.or_texture_pixel_offset(t, x, y, mip) == expected, (x, y, mip)
            checked += 1
        for x, y, mip, value in block["writes"]:
            l.or_texture_write_pixel(t, x, y, mip, value)
        for x, y, mip, expected in block["read"]:
            assert l.or_texture_read_pixel(t, x, y, mip) == expected, (x, y, mip)
            checked += 1
        for u, v, mip, expected in block["nearest"]:
            assert l.or_sample_nearest(t, C.c_float(u), C.c_float(v), mip, 0) == expected, (u, v, mip)
            checked += 1
    mix = data["linear_mix"]
    for a, b, w, e in zip(mix["a"], mix["b"], mix["weight"], mix["expected"]):
        assert port.lib().or_interpolate_color_linear(a, b, w) == e
        checked += 1
    assert checked > 400


def fixture_scene(path):
    from dfpsr_gb300 import scenes
    z = np.load(path)
    s = scenes.Scene(int(z["width"]), int(z["height"]), z["positions"], z["poly_indices"], z["tex_coords"], z["colors"],
                     z["diffuse"] if "diffuse" in z else None, int(z["diffuse_levels"]),
                     z["light"] if "light" in z else None, int(z["light_levels"]), int(z["filter"]),
                     z["camera_location"], bool(z["perspective"]), float(z["slope"]), float(z["near_clip"]),
                     float(z["far_clip"]), z["model_to_world"])
    return s, z


FIXTURES = sorted(glob.glob(os.path.join(GOLDEN, "render_*.npz")))


@pytest.mark.parametrize("path", FIXTURES, ids=[os.path.basename(p)[7:-4] for p in FIXTURES])
def test_oracle_matches_reference_renders(built, path):
    from oracle import port
    scene, z = fixture_scene(path)
    color, depth, _ = port.render(scene)
    assert np.array_equal(color, z["color"])
    assert np.array_equal(depth.view(np.uint32), z["depth"].view(np.uint32))
    bgra, _, _ = port.render(scene, pack_order=1)
    assert np.array_equal(bgra, z["color_bgra"])
    depth_only, _ = port.render_depth(scene)
    assert np.array_equal(depth_only.view(np.uint32), z["depth_only"].view(np.uint32))


@pytest.mark.gpu
@pytest.mark.parametrize("path", FIXTURES, ids=[os.path.basename(p)[7:-4] for p in FIXTURES])
def test_gpu_matches_reference_renders(ctx, path):
    import dfpsr_gb300 as d
    scene, z = fixture_scene(path)
    model = d.Model(ctx, scene)
    color, depth = d.render_scene(ctx, scene, model=model)
    assert np.array_equal(color, z["color"])
    assert np.array_equal(depth.view(np.uint32), z["depth"].view(np.uint32))
    bgra, _ = d.render_scene(ctx, scene, pack_order=1, model=model)
    assert np.array_equal(bgra, z["color_bgra"])
    depth_only = np.zeros((scene.height, scene.width), np.float32)
    ctx.render_depth(model, model.camera, depth_only)
    assert np.array_equal(depth_only.view(np.uint32), z["depth_only"].view(np.uint32))


@pytest.mark.gpu
def test_gpu_texture_fields_match_known_answers(ctx):
    import dfpsr_gb300 as d
    for block in kats()["textures"]:
        w, h = 1 << block["log2w"], 1 << block["log2h"]
        fields, _ = d.Texture(ctx, np.zeros((h, w), np.uint32), block["maxMip"] + 1).read()
        got = dict(zip(FIELD_ORDER, fields.tolist()))
        for name in ("startOffset", "maxLevelMask"):
            if name in block["fields"]:
                assert got[name] == block["fields"][name]


def test_oracle_occlusion_sessions(built):
    """The oracle plays the occlusion-grid sessions the reference played for the fixture."""
    import sys
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    import make_golden
    import occlusion_script as o
    from dfpsr_gb300 import scenes
    with open(os.path.join(GOLDEN, "occlusion_sessions.json")) as f:
        sessions = json.load(f)
    assert len(sessions) == 8
    for name, expect in sessions.items():
        sc = scenes.occlusion_scene(**expect["params"])
        assert make_golden.scene_digest(sc) == expect["inputs"], f"{name}: the seeded inputs changed"
        got = o.play(o.OracleEngine(), sc, use_color=expect["use_color"], use_depth=expect["use_depth"], debug=expect["debug"])
        assert got["visible"] == expect["visible"], name
        assert got["has_occluders"] == expect["has_occluders"], name
        frames = [[make_golden.image_digest(f[0]), make_golden.image_digest(f[1])] for f in got["frames"]]
        assert frames == expect["frames"], name


def test_oracle_texture_resize_matches_reference_fixture(built):
    """Images whose sizes are not powers of two: filter_resize (linear) to the next powers of two,
    then the pyramid, as the reference made them."""
    import hashlib
    import sys
    sys.path.insert(0, GOLDEN)
    import make_golden
    from oracle import port
    with open(os.path.join(GOLDEN, "texture_resize.json")) as f:
        cases = json.load(f)
    assert len(cases) == len(make_golden.TEXTURE_RESIZE_CASES)
    for case in cases:
        t = port.OracleTexture(make_golden.texture_resize_image(case["width"], case["height"]), case["resolutions"])
        assert list(t.t.fields()) == case["fields"], case
        assert hashlib.sha256(t.t.array().tobytes()).hexdigest() == case["pyramid"], case


def test_oracle_dense_render_matches_reference_fixture(built):
    """renderDenseModel: the oracle leaves the images the reference left (tests/golden/dense_render.json)."""
    import sys
    sys.path.insert(0, GOLDEN)
    import make_golden
    from dfpsr_gb300 import scenes
    from oracle import port
    with open(os.path.join(GOLDEN, "dense_render.json")) as f:
        cases = json.load(f)
    assert len(cases) == len(make_golden.DENSE_CASES)
    for case in cases:
        sc = scenes.dense_scene(seed=case["seed"], view_index=case["view_index"], prefilled=case["prefilled"])
        inputs = np.concatenate([sc.positions.reshape(-1), sc.colors.reshape(-1), sc.model_to_world, sc.height.reshape(-1)])
        assert make_golden.image_digest(inputs.view(np.uint32)) == case["inputs"], "the seeded scene generator changed"
        view = port.ortho_view(sc.camera_tilt, sc.pixels_per_tile, sc.view_index)
        h, d, n = port.dense_render(port.dense_model(sc.positions, sc.polygons, sc.colors), view, sc.height, sc.diffuse,
                                    sc.normal, sc.origin, sc.model_to_world, case["high_quality"])
        assert make_golden.image_digest(h.view(np.uint32)) == case["height"], case
        assert make_golden.image_digest(d) == case["diffuse"], case
        assert make_golden.image_digest(n) == case["normal"], case
