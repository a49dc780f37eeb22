"""The oracle against the reference itself, run here where the reference was built from its
sources (skipped elsewhere): bit-exact against the exact (scalar, no-FMA) build on seeded
scenes, including the full 800x600 random-triangle configuration and the threaded renderer."""
import numpy as np
import pytest

from dfpsr_gb300 import scenes


@pytest.fixture(scope="module")
def ref_lib(built):
    from oracle import ref
    if not ref.available("exact"):
        pytest.skip("the reference was not built from source on this machine")
    return ref


CASES = {
    "random_800x600": lambda: scenes.random_triangles(seed=1234),
    "terrain_grid128": lambda: scenes.terrain(seed=3, grid=128, width=640, height=360, texture_size=256),
    "clipping": lambda: _clipping(),
    "orthogonal": lambda: _ortho(),
    "lightmap": lambda: scenes.with_variant(scenes.random_triangles(seed=8, triangles=1500, width=256, height=192), light=True),
}


def _clipping():
    s = scenes.random_triangles(seed=9, triangles=3000, width=400, height=300)
    s.camera_location = scenes.camera_location((0.1, 0.2, -0.3), (0.0, 0.0, 1.0))
    return s


def _ortho():
    s = scenes.random_triangles(seed=23, triangles=1500, width=256, height=200)
    s.perspective = False
    s.slope = 1.3
    return s


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_equals_reference_exact_build(ref_lib, name):
    from oracle import port
    scene = CASES[name]()
    model = ref_lib.RefModel(scene, "exact")
    rc, rd = model.render()
    oc, od, _ = port.render(scene)
    assert np.array_equal(rc, oc)
    assert np.array_equal(rd.view(np.uint32), od.view(np.uint32))
    tc, td = model.render(threaded=True)
    bc, bd, _ = port.render(scene, bands=12, threads=4)
    assert np.array_equal(tc, bc) and np.array_equal(td.view(np.uint32), bd.view(np.uint32))
    depth_ref = model.render_depth()
    depth_oracle, _ = port.render_depth(scene)
    assert np.array_equal(depth_ref.view(np.uint32), depth_oracle.view(np.uint32))


def test_row_intervals_equal_reference(ref_lib):
    """rasterizeTriangle's row intervals (ITriangle2D.cpp:150-176) for random and extreme triangles."""
    from oracle import port
    r = np.random.default_rng(77)
    for i in range(3000):
        f = r.integers(-200 * 256, 1000 * 256, 6).astype(np.int64)
        if i % 3 == 1:
            f[1] = f[3] + r.integers(-2, 3)
        clip = [0, 0, 800, 600]
        a = ref_lib.triangle_rows(f, clip)
        b = port.triangle_rows(f, clip)
        assert a[0] == b[0] or len(a[1]) == 0
        assert np.array_equal(a[1], b[1]) and np.array_equal(a[2], b[2])


@pytest.mark.parametrize("perspective", [True, False])
@pytest.mark.parametrize("targets", [(True, True), (True, False), (False, True)])
@pytest.mark.parametrize("debug", [False, True])
def test_oracle_occlusion_session_equals_reference(ref_lib, perspective, targets, debug):
    """renderer_occludeFromBox / FromExistingTriangles / FromTopRows, isBoxVisible, hasOccluders and
    renderer_end with completeOcclusion, two frames on one renderer (tests/occlusion_script.py);
    with debug, the silhouettes and the wireframe overlay."""
    import occlusion_script as o
    sc = scenes.occlusion_scene(perspective=perspective)
    a = o.play(o.OracleEngine(), sc, use_color=targets[0], use_depth=targets[1], debug=debug)
    b = o.play(o.RefEngine(), sc, use_color=targets[0], use_depth=targets[1], debug=debug)
    o.assert_same(a, b, f"perspective {perspective} targets {targets}")
    assert 0 < sum(a["visible"]) < len(a["visible"])  # some boxes occluded, some not


def test_oracle_texture_resize_equals_reference(ref_lib):
    """filter_resize (Sampler::Linear) inside texture_create_RgbaU8: upscaling in both directions
    (two steps), downscaling (the bilinear reference path), one dimension only (the vertical and
    horizontal paths), tiny and large images."""
    from oracle import port
    lib = ref_lib._load("exact")
    rng = np.random.default_rng(5)
    for w, h in [(1, 1), (3, 5), (5, 3), (17, 16), (16, 17), (20, 12), (100, 60), (60, 100), (64, 48), (48, 64),
                 (255, 257), (129, 31), (1000, 600), (33, 2), (2, 33), (513, 1)]:
        img = rng.integers(0, 2**32, size=(h, w), dtype=np.uint64).astype(np.uint32)
        for levels in (1, 4, 16):
            t = port.OracleTexture(img, levels)
            fields, pixels = ref_lib.RefTexture(lib, img, levels).info()
            assert list(t.t.fields()) == list(fields), (w, h, levels)
            assert np.array_equal(t.t.array(), pixels), (w, h, levels)


def test_oracle_draw_line_equals_reference(ref_lib):
    """draw_line (api/drawAPI.cpp:176-279) on random segments, partly or wholly outside the image."""
    from oracle import port
    rng = np.random.default_rng(3)
    for _ in range(2000):
        w, h = int(rng.integers(1, 40)), int(rng.integers(1, 40))
        img = rng.integers(0, 2**32, size=(h, w), dtype=np.uint64).astype(np.uint32)
        x1, y1, x2, y2 = [int(v) for v in rng.integers(-20, 60, 4)]
        color = int(rng.integers(0, 2**32))
        assert np.array_equal(port.draw_line(img, x1, y1, x2, y2, color), ref_lib.draw_line(img, x1, y1, x2, y2, color))


def _odd(w, h, n, seed=11, **kw):
    import dataclasses
    s = scenes.random_triangles(seed=seed, triangles=n, width=w, height=h, texture_size=32)
    if kw.get("ortho"):
        s.perspective = False
        s.slope = 1.3
    if kw.get("alpha"):
        s = dataclasses.replace(s, filter=1)
    return s


ODD_CASES = {
    "1x57": lambda: _odd(1, 57, 300),
    "64x1": lambda: _odd(64, 1, 300),
    "97x3": lambda: _odd(97, 3, 400),
    "199x151": lambda: _odd(199, 151, 2000),
    "199x151_ortho": lambda: _odd(199, 151, 2000, seed=12, ortho=True),
    "199x151_alpha": lambda: _odd(199, 151, 1500, seed=13, alpha=True),
    "48x33_dense": lambda: _odd(48, 33, 3000, seed=14),
    "800x601": lambda: scenes.random_triangles(seed=1234, width=800, height=601),
}


@pytest.mark.parametrize("name", sorted(ODD_CASES))
def test_oracle_equals_reference_odd_heights(ref_lib, name):
    """Targets of odd height: the last row pair's missing lower row points at the upper row, so
    the run of full quads writes its lower lanes there (fillerTemplates.h:285-306).  Prefilled
    targets, colour-only and depth-only targets and the threaded renderer, bit for bit."""
    from oracle import port
    scene = ODD_CASES[name]()
    h, w = scene.height, scene.width
    model = ref_lib.RefModel(scene, "exact")
    rng = np.random.default_rng(7)
    color0 = rng.integers(0, 2**32, size=(h, w), dtype=np.uint64).astype(np.uint32)
    depth0 = rng.uniform(0.0, 0.3, size=(h, w)).astype(np.float32)
    for kw in (dict(), dict(color=color0, depth=depth0), dict(use_depth=False), dict(use_color=False)):
        rc, rd = model.render(**kw)
        oc, od, _ = port.render(scene, **kw)
        if rc is not None:
            assert np.array_equal(rc, oc), (name, kw.keys(), int((rc != oc).sum()))
        if rd is not None:
            assert np.array_equal(rd.view(np.uint32), od.view(np.uint32)), (name, kw.keys())
    tc, td = model.render(threaded=True)
    bc, bd, _ = port.render(scene, bands=12, threads=4)
    assert np.array_equal(tc, bc) and np.array_equal(td.view(np.uint32), bd.view(np.uint32))


def _mixed_frame_tasks():
    """Tasks of one frame in order: perspective solid, orthogonal solid, perspective alpha,
    orthogonal alpha, perspective solid (each task with its own camera)."""
    import dataclasses
    out = []
    for i, (perspective, alpha) in enumerate([(True, False), (False, False), (True, True), (False, True), (True, False)]):
        s = scenes.random_triangles(seed=140 + i, triangles=700, width=211, height=143, texture_size=32)
        if not perspective:
            s.perspective = False
            s.slope = 1.3
        if alpha:
            s = dataclasses.replace(s, filter=1)
        s.model_to_world = np.array([0.1 * i, -0.05 * i, 0.2 * i, 1, 0, 0, 0, 1, 0, 0, 0, 1], np.float32)
        out.append(s)
    return out


def test_oracle_equals_reference_on_frames_mixing_projections_and_filters(ref_lib):
    """renderer_giveTask with perspective and orthogonal cameras and solid and alpha-filtered models
    in one frame: every triangle tests depth with its own projection's comparison
    (fillerTemplates.h:108-152) in submission order."""
    from oracle import port
    tasks = _mixed_frame_tasks()
    h, w = tasks[0].height, tasks[0].width
    rng = np.random.default_rng(3)
    color0 = rng.integers(0, 2**32, size=(h, w), dtype=np.uint64).astype(np.uint32)
    depth0 = rng.uniform(0.0, 0.3, size=(h, w)).astype(np.float32)
    r = ref_lib.RefRenderer()
    o = port.OracleRenderer()
    for eng in (r, o):
        eng.begin(color0, depth0)
    models = [ref_lib.RefModel(s) for s in tasks]
    pms = [port.PreparedModel(s) for s in tasks]
    for s, m, pm in zip(tasks, models, pms):
        r.give_task(m, s.model_to_world, pm.cam)
        o.give_task(pm, s.model_to_world, pm.cam)
    rc, rd = r.end(False)
    oc, od, _ = o.end()
    assert np.array_equal(rc, oc)
    assert np.array_equal(rd.view(np.uint32), od.view(np.uint32))
    assert (rc != color0).sum() > 1000


def test_oracle_texture_from_other_pack_orders_equals_reference(ref_lib):
    """texture_create_RgbaU8 of BGRA, ARGB and ABGR images: the copy and the horizontal and bilinear
    paths unpack the source's order, the aligned vertical-only path mixes its bytes as they lie
    (filterAPI.cpp:157-260), a two-step upscale unpacks in its first step."""
    from oracle import port
    lib = ref_lib._load("exact")
    rng = np.random.default_rng(15)
    for w, h in [(16, 16), (16, 10), (16, 20), (10, 16), (20, 16), (12, 20), (100, 60), (60, 100), (33, 2), (2, 33), (5, 3)]:
        img = rng.integers(0, 2**32, size=(h, w), dtype=np.uint64).astype(np.uint32)
        for order in (1, 2, 3):
            for levels in (1, 16):
                t = port.OracleTexture(img, levels, pack_order=order)
                fields, pixels = ref_lib.RefTexture(lib, img, levels, pack_order=order).info()
                assert list(t.t.fields()) == list(fields), (w, h, order, levels)
                assert np.array_equal(t.t.array(), pixels), (w, h, order, levels)
