"""GPU parity of the sprite engine's dense models (DenseModel_create and renderDenseModel,
SDK/SpriteEngine/spriteAPI.cpp:1156-1327) against the oracle (which tests/test_dense_cpu.py pins
to the reference): height, diffuse and normal images bit for bit, in both qualities, every view
direction, over empty and prefilled images, partly outside the image, and several instances drawn
one after another into the same images."""
import numpy as np
import pytest

from dfpsr_gb300 import scenes

pytestmark = pytest.mark.gpu


def _gpu(ctx, sc, model, high_quality, height=None, diffuse=None, normal=None, origin=None, transform=None):
    import torch
    import dfpsr_gb300 as d
    dev = lambda a, dt: torch.tensor(np.ascontiguousarray(a).view(dt), device="cuda")
    h = dev(sc.height if height is None else height, np.float32)
    di = dev(sc.diffuse if diffuse is None else diffuse, np.int32)
    n = dev(sc.normal if normal is None else normal, np.int32)
    view = d.ortho_view(sc.camera_tilt, sc.pixels_per_tile, sc.view_index)
    ctx.dense_render(model, view, h, di, n, sc.origin if origin is None else origin,
                     sc.model_to_world if transform is None else transform, high_quality)
    return h.cpu().numpy(), di.cpu().numpy().view(np.uint32), n.cpu().numpy().view(np.uint32)


def _oracle(sc, tris, high_quality, height=None, diffuse=None, normal=None, origin=None, transform=None):
    from oracle import port
    view = port.ortho_view(sc.camera_tilt, sc.pixels_per_tile, sc.view_index)
    return port.dense_render(tris, view, sc.height if height is None else height, sc.diffuse if diffuse is None else diffuse,
                             sc.normal if normal is None else normal, sc.origin if origin is None else origin,
                             sc.model_to_world if transform is None else transform, high_quality)


def _same(a, b, label):
    (h, d, n), (rh, rd, rn) = a, b
    assert np.array_equal(h.view(np.uint32), rh.view(np.uint32)), f"{label}: height differs at {int((h.view(np.uint32) != rh.view(np.uint32)).sum())} pixels"
    assert np.array_equal(d, rd), f"{label}: {int((d != rd).sum())} diffuse pixels differ"
    assert np.array_equal(n, rn), f"{label}: {int((n != rn).sum())} normal pixels differ"


@pytest.mark.parametrize("high_quality", [False, True])
@pytest.mark.parametrize("view_index,prefilled", [(0, False), (1, True), (2, False), (3, True), (4, False), (5, True),
                                                   (6, False), (7, True)])
def test_dense_render_matches_oracle(ctx, high_quality, view_index, prefilled):
    import dfpsr_gb300 as d
    from oracle import port
    sc = scenes.dense_scene(seed=40 + view_index, view_index=view_index, prefilled=prefilled)
    model = d.DenseModel(ctx, sc.positions, sc.polygons, sc.colors)
    tris = port.dense_model(sc.positions, sc.polygons, sc.colors)
    got = _gpu(ctx, sc, model, high_quality)
    _same(got, _oracle(sc, tris, high_quality), f"view {view_index} hq {high_quality}")
    assert int((got[1] != sc.diffuse).sum()) > 1000
    model.destroy()


def test_dense_instances_in_sequence_and_at_the_edges(ctx):
    """Several placements of two dense models drawn one after another into the same images (the
    sprite world's drawModel per instance), some crossing the image's edges."""
    import dfpsr_gb300 as d
    from oracle import port
    a = scenes.dense_scene(seed=51, width=320, height=200, prefilled=True)
    b = scenes.dense_scene(seed=52, width=320, height=200, major=12, minor=6)
    models = [(d.DenseModel(ctx, s.positions, s.polygons, s.colors), port.dense_model(s.positions, s.polygons, s.colors), s)
              for s in (a, b)]
    rng = np.random.default_rng(3)
    h, di, n = a.height, a.diffuse, a.normal
    rh, rd, rn = h, di, n
    for k in range(6):
        model, tris, s = models[k % 2]
        origin = (float(rng.uniform(-20, 340)), float(rng.uniform(-20, 220)))
        transform = np.concatenate([rng.uniform(-1, 1, 3), scenes.random_rotation(rng).reshape(-1)]).astype(np.float32)
        h, di, n = _gpu(ctx, a, model, k % 3 == 0, h, di, n, origin, transform)
        rh, rd, rn = _oracle(a, tris, k % 3 == 0, rh, rd, rn, origin, transform)
        _same((h, di, n), (rh, rd, rn), f"instance {k}")
    for m, _, _ in models:
        m.destroy()


def test_dense_model_errors(ctx):
    import torch
    import dfpsr_gb300 as d
    sc = scenes.dense_scene(seed=53, width=32, height=32)
    model = d.DenseModel(ctx, sc.positions, sc.polygons, sc.colors)
    view = d.ortho_view(sc.camera_tilt, sc.pixels_per_tile, 0)
    host = np.zeros((32, 32), np.float32)
    rgba = torch.zeros((32, 32), dtype=torch.int32, device="cuda")
    with pytest.raises(d.DsrgError) as e:
        ctx.dense_render(model, view, host, rgba, rgba, sc.origin, sc.model_to_world)  # the height image is on the host
    assert e.value.status == 1  # DSRG_ERROR_INVALID_ARGUMENT
    with pytest.raises(d.DsrgError):
        d.DenseModel(ctx, sc.positions, np.array([[0, 1, 10**6, -1]], np.int32), sc.colors[:1])
    empty = d.DenseModel(ctx, sc.positions, np.zeros((0, 4), np.int32), np.zeros((0, 4, 4), np.float32))
    h = torch.full((32, 32), -5.0, device="cuda")
    ctx.dense_render(empty, view, h, rgba, rgba, sc.origin, sc.model_to_world)
    assert float(h.min()) == -5.0
    model.destroy()
    empty.destroy()


def test_dense_render_matches_reference_fixture(ctx):
    """The GPU leaves the images the reference left (tests/golden/dense_render.json)."""
    import json
    import os
    import sys
    import dfpsr_gb300 as d
    from conftest import ROOT
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    import make_golden
    with open(os.path.join(ROOT, "tests", "golden", "dense_render.json")) as f:
        cases = json.load(f)
    for case in cases:
        sc = scenes.dense_scene(seed=case["seed"], view_index=case["view_index"], prefilled=case["prefilled"])
        model = d.DenseModel(ctx, sc.positions, sc.polygons, sc.colors)
        h, di, n = _gpu(ctx, sc, model, case["high_quality"])
        assert make_golden.image_digest(h.view(np.uint32)) == case["height"], case
        assert make_golden.image_digest(di) == case["diffuse"], case
        assert make_golden.image_digest(n) == case["normal"], case
        model.destroy()


@pytest.mark.parametrize("high_quality", [False, True])
def test_dense_render_many_equals_calls_in_sequence(ctx, high_quality):
    """One call for a sequence of instances of two models (some overlapping, some crossing the
    edges, one outside) leaves what the same instances drawn one call after another leave, and
    what the oracle leaves."""
    import torch
    import dfpsr_gb300 as d
    from oracle import port
    a = scenes.dense_scene(seed=71, width=300, height=220, prefilled=True)
    b = scenes.dense_scene(seed=72, width=300, height=220, major=12, minor=6)
    models = [(d.DenseModel(ctx, s.positions, s.polygons, s.colors), port.dense_model(s.positions, s.polygons, s.colors)) for s in (a, b)]
    rng = np.random.default_rng(9)
    instances = []
    for k in range(10):
        origin = (float(rng.uniform(-30, 330)), float(rng.uniform(-30, 250))) if k != 7 else (5000.0, 5000.0)
        transform = np.concatenate([rng.uniform(-0.5, 0.5, 3), scenes.random_rotation(rng).reshape(-1)]).astype(np.float32)
        instances.append((k % 2, origin, transform))
    view = d.ortho_view(a.camera_tilt, a.pixels_per_tile, a.view_index)
    dev = lambda arr, dt: torch.tensor(np.ascontiguousarray(arr).view(dt), device="cuda")
    h, di, n = dev(a.height, np.float32), dev(a.diffuse, np.int32), dev(a.normal, np.int32)
    ctx.dense_render_many([(models[m][0], o, t) for m, o, t in instances], view, h, di, n, high_quality)
    got = (h.cpu().numpy(), di.cpu().numpy().view(np.uint32), n.cpu().numpy().view(np.uint32))
    h2, d2, n2 = dev(a.height, np.float32), dev(a.diffuse, np.int32), dev(a.normal, np.int32)
    for m, o, t in instances:
        ctx.dense_render(models[m][0], view, h2, d2, n2, o, t, high_quality)
    seq = (h2.cpu().numpy(), d2.cpu().numpy().view(np.uint32), n2.cpu().numpy().view(np.uint32))
    rh, rd, rn = a.height, a.diffuse, a.normal
    for m, o, t in instances:
        rh, rd, rn = _oracle(a, models[m][1], high_quality, rh, rd, rn, o, t)
    _same(got, (rh, rd, rn), "many vs oracle")
    _same(seq, (rh, rd, rn), "calls vs oracle")
    for m, _ in models:
        m.destroy()


def test_benchmarked_dense_instances_full_size(ctx):
    """The benchmarked dense-model sequence itself: 64 placements of a 3,200-triangle torus at
    1920x1080 in one dsrg_dense_render_many call, against the oracle's 64 renderDenseModel calls."""
    import torch
    import dfpsr_gb300 as d
    from dfpsr_gb300 import scenes
    from oracle import port
    sc = scenes.dense_scene(seed=77, width=1920, height=1080, major=80, minor=20, pixels_per_tile=64)
    rng = np.random.default_rng(5)
    places = [((float(rng.uniform(0, 1920)), float(rng.uniform(0, 1080))),
               np.concatenate([rng.uniform(-1, 1, 3), scenes.random_rotation(rng).reshape(-1)]).astype(np.float32))
              for _ in range(64)]
    model = d.DenseModel(ctx, sc.positions, sc.polygons, sc.colors)
    view = d.ortho_view(sc.camera_tilt, sc.pixels_per_tile, sc.view_index)
    h = torch.tensor(sc.height, device="cuda")
    di = torch.zeros((1080, 1920), dtype=torch.int32, device="cuda")
    n = torch.zeros_like(di)
    ctx.dense_render_many([(model, origin, transform) for origin, transform in places], view, h, di, n, False)
    tris = port.dense_model(sc.positions, sc.polygons, sc.colors)
    pv = port.ortho_view(sc.camera_tilt, sc.pixels_per_tile, sc.view_index)
    rh, rd, rn = sc.height, np.zeros((1080, 1920), np.uint32), np.zeros((1080, 1920), np.uint32)
    for origin, transform in places:
        rh, rd, rn = port.dense_render(tris, pv, rh, rd, rn, origin, transform, False)
    assert np.array_equal(h.cpu().numpy().view(np.uint32), rh.view(np.uint32))
    assert np.array_equal(di.cpu().numpy().view(np.uint32), rd)
    assert np.array_equal(n.cpu().numpy().view(np.uint32), rn)
    assert (rd != 0).sum() > 10000
    model.destroy()
