"""GPU parity of the renderer's occlusion grid against the oracle (which the CPU tests pin to the
reference): box occluders, occluders from existing triangles (a triangle-setup pass on the GPU),
from the depth image's top rows (a GPU kernel), box tests, whole models skipped at
renderer_give_task, and draw commands skipped by completeOcclusion inside the GPU triangle setup.
The session is tests/occlusion_script.py; images, box-test answers, the grid after every
occluder and the fragment counts must all be identical."""
import os

import numpy as np
import pytest

from dfpsr_gb300 import scenes

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("perspective", [True, False])
@pytest.mark.parametrize("targets", [(True, True), (True, False), (False, True)])
@pytest.mark.parametrize("debug", [False, True])
def test_occlusion_session_matches_oracle(ctx, perspective, targets, debug):
    """With debug, also the silhouettes of occludeFromBox and renderer_end's wireframe overlay."""
    import occlusion_script as o
    sc = scenes.occlusion_scene(perspective=perspective)
    a = o.play(o.GpuEngine(ctx), sc, use_color=targets[0], use_depth=targets[1], debug=debug)
    b = o.play(o.OracleEngine(), sc, use_color=targets[0], use_depth=targets[1], debug=debug)
    o.assert_same(a, b, f"perspective {perspective} targets {targets} debug {debug}")


def test_wireframe_of_a_large_frame_with_alpha_runs(ctx):
    """The wireframe of a frame of solid and alpha-filtered runs (lines gathered from every run's
    commands), at 1080p with long edges leaving the image."""
    import dataclasses
    import dfpsr_gb300 as d
    from oracle import port
    base = scenes.random_triangles(seed=91, triangles=3000, width=1920, height=1080, texture_size=64)
    base.camera_location = scenes.camera_location((0.1, 0.2, -1.2), (0.0, 0.0, 1.0))
    parts = [dataclasses.replace(base, filter=f) for f in (0, 1)]
    parts[1] = dataclasses.replace(parts[1], model_to_world=np.array([0.3, 0.1, 0.2, 1, 0, 0, 0, 1, 0, 0, 0, 1], np.float32))
    o = port.OracleRenderer()
    color = np.zeros((1080, 1920), np.uint32)
    depth = np.zeros((1080, 1920), np.float32)
    o.begin(color, depth)
    pms = [port.PreparedModel(p) for p in parts]
    for pm, p in zip(pms, parts):
        o.give_task(pm, p.model_to_world, pm.cam)
    rc, rz, _ = o.end(debug_wireframe=True)
    r = d.Renderer(ctx)
    c, z = color.copy(), depth.copy()
    r.begin(c, z)
    models = [d.Model(ctx, p) for p in parts]
    for m, p in zip(models, parts):
        r.give_task(m, m.camera, p.model_to_world)
    r.end(debug_wireframe=True)
    assert np.array_equal(c, rc), f"{int((c != rc).sum())} pixels differ"
    assert np.array_equal(z.view(np.uint32), rz.view(np.uint32))
    r.destroy()


def test_occlusion_sessions_match_reference_fixtures(ctx):
    import json
    import sys
    from conftest import ROOT
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    import make_golden
    import occlusion_script as o
    with open(os.path.join(ROOT, "tests", "golden", "occlusion_sessions.json")) as f:
        sessions = json.load(f)
    for name, expect in sessions.items():
        sc = scenes.occlusion_scene(**expect["params"])
        got = o.play(o.GpuEngine(ctx), sc, use_color=expect["use_color"], use_depth=expect["use_depth"], debug=expect["debug"])
        assert got["visible"] == expect["visible"], name
        frames = [[make_golden.image_digest(f[0]), make_golden.image_digest(f[1])] for f in got["frames"]]
        assert frames == expect["frames"], name


def test_occlusion_culls_and_keeps_alpha_runs(ctx):
    """An alpha-filtered model in an occluded frame: completeOcclusion applies to every run, and
    alpha-filtered triangles never occlude."""
    import dataclasses
    import occlusion_script as o
    sc = scenes.occlusion_scene(seed=79, props=8)
    glass = dataclasses.replace(sc.field, filter=1)
    results = []
    for engine in (o.GpuEngine(ctx), o.OracleEngine()):
        cam = engine.camera(sc.camera)
        engine.begin(sc.color, sc.depth)
        engine.box(sc.wall, cam)
        engine.give(sc.wall, cam)
        engine.give(glass, cam)
        engine.existing()
        grid = engine.grid()
        for p in sc.props:
            engine.give(p, cam)
        results.append((grid, engine.end()))
    (ga, fa), (gb, fb) = results
    assert np.array_equal(ga.view(np.uint32), gb.view(np.uint32))
    assert np.array_equal(fa[0], fb[0]) and np.array_equal(fa[1].view(np.uint32), fb[1].view(np.uint32))
    assert fa[2] == fb[2]


def test_occlusion_errors(ctx):
    import dfpsr_gb300 as d
    r = d.Renderer(ctx)
    cam = d.camera_struct(scenes.occlusion_scene().camera)
    box = (np.zeros(3, np.float32), np.ones(3, np.float32), scenes.IDENTITY)
    with pytest.raises(d.DsrgError) as e:
        r.occlude_from_box(*box, cam)
    assert e.value.status == 4
    with pytest.raises(d.DsrgError):
        r.is_box_visible(*box, cam)
    with pytest.raises(d.DsrgError):
        r.occlude_from_existing_triangles()
    color = np.zeros((32, 32), np.uint32)
    r.begin(color, None)
    with pytest.raises(d.DsrgError) as e:
        r.occlude_from_top_rows(cam)  # no depth image
    assert e.value.status == 4
    assert r.has_occluders  # the grid was prepared before the check, as in the reference
    r.end()
    r.destroy()
