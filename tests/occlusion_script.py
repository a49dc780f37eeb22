"""One renderer session with the occlusion grid, played on three engines: the CPU oracle, the
reference itself (when it was built here) and the GPU library.  Each engine receives the same
calls in the same order, and the session records what a caller can observe: every
renderer_isBoxVisible answer, renderer_hasOccluders, the final images and (oracle and GPU) the
grid after each occluder and the fragment count.

Frame 1: a box occluder, box tests, the wall, a tilted panel and the field given, occluders from
the existing triangles, half of the props given (several culled whole by their box), occluders from the depth
image's top rows, box tests and the other props.  Frame 2 (same renderer): box tests before any
occluder (they read the grid the first frame left), then top rows and every model again.
"""
from __future__ import annotations

import numpy as np

from dfpsr_gb300 import scenes


class OracleEngine:
    name = "oracle"

    def __init__(self):
        from oracle import port
        self.port = port
        self.r = port.OracleRenderer()
        self.models = {}

    def model(self, s):
        if id(s) not in self.models:
            self.models[id(s)] = self.port.PreparedModel(s)
        return self.models[id(s)]

    def camera(self, s):
        return self.port.camera_desc(s)

    def begin(self, color, depth):
        self.r.begin(color, depth)

    def give(self, s, cam):
        self.r.give_task(self.model(s), s.model_to_world, cam)

    def box(self, s, cam, debug=False):
        mn, mx = scenes.OcclusionScene.bound(s)
        self.r.occlude_from_box(mn, mx, s.model_to_world, cam, debug)

    def existing(self):
        self.r.occlude_from_existing_triangles()

    def top_rows(self, cam):
        assert self.r.occlude_from_top_rows(bool(cam.perspective)) == 0

    def visible(self, s, cam):
        mn, mx = scenes.OcclusionScene.bound(s)
        return self.r.is_box_visible(mn, mx, s.model_to_world, cam)

    def has_occluders(self):
        return self.r.has_occluders()

    def grid(self):
        return self.r.grid()

    def end(self, wireframe=False):
        c, d, info = self.r.end(coverage=False, debug_wireframe=wireframe)
        return c, d, info["fragments"]


class RefEngine(OracleEngine):
    name = "reference"

    def __init__(self):
        from oracle import port, ref
        self.port, self.ref = port, ref
        self.r = ref.RefRenderer()
        self.models = {}

    def model(self, s):
        if id(s) not in self.models:
            self.models[id(s)] = self.ref.RefModel(s)
        return self.models[id(s)]

    def top_rows(self, cam):
        self.r.occlude_from_top_rows(cam)

    def grid(self):
        return None

    def end(self, wireframe=False):
        c, d = self.r.end(wireframe)
        return c, d, None


class GpuEngine(OracleEngine):
    name = "gpu"

    def __init__(self, ctx):
        import dfpsr_gb300 as d
        self.d, self.ctx = d, ctx
        self.r = d.Renderer(ctx)
        self.models = {}
        self.images = None

    def model(self, s):
        if id(s) not in self.models:
            self.models[id(s)] = self.d.Model(self.ctx, s)
        return self.models[id(s)]

    def camera(self, s):
        return self.d.camera_struct(s)

    def begin(self, color, depth):
        self.images = (None if color is None else np.array(color, np.uint32), None if depth is None else np.array(depth, np.float32))
        self.r.begin(*self.images)

    def give(self, s, cam):
        self.r.give_task(self.model(s), cam, s.model_to_world)

    def box(self, s, cam, debug=False):
        mn, mx = scenes.OcclusionScene.bound(s)
        self.r.occlude_from_box(mn, mx, s.model_to_world, cam, debug)

    def existing(self):
        self.r.occlude_from_existing_triangles()

    def top_rows(self, cam):
        self.r.occlude_from_top_rows(cam)

    def visible(self, s, cam):
        mn, mx = scenes.OcclusionScene.bound(s)
        return self.r.is_box_visible(mn, mx, s.model_to_world, cam)

    def has_occluders(self):
        return self.r.has_occluders

    def grid(self):
        return self.r.occlusion_grid()

    def end(self, wireframe=False):
        self.ctx.set_counting(True, None)
        try:
            self.r.end(wireframe)
            fragments = self.ctx.stats()["fragments"]
        finally:
            self.ctx.set_counting(False)
        return self.images[0], self.images[1], fragments


def play(engine, sc: scenes.OcclusionScene, *, use_color: bool = True, use_depth: bool = True, debug: bool = False) -> dict:
    """debug: the box occluder keeps its silhouette, frame 1 ends with the wireframe overlay, and
    frame 2 draws a second silhouette (and the first one again when frame 1 had no colour image)."""
    cam = engine.camera(sc.camera)
    out = {"visible": [], "has_occluders": [], "grids": [], "frames": []}
    color = sc.color if use_color else None
    depth = sc.depth if use_depth else None
    props = sc.props
    # frame 1
    engine.begin(color, depth)
    out["has_occluders"].append(engine.has_occluders())
    engine.box(sc.wall, cam, debug)
    out["grids"].append(engine.grid())
    out["visible"] += [engine.visible(p, cam) for p in props]
    engine.give(sc.wall, cam)
    engine.give(sc.panel, cam)
    engine.give(sc.field, cam)
    engine.existing()
    out["grids"].append(engine.grid())
    for p in props[0::2]:
        engine.give(p, cam)
    if use_depth:
        engine.top_rows(cam)
        out["grids"].append(engine.grid())
    out["visible"] += [engine.visible(p, cam) for p in props[1::2]]
    for p in props[1::2]:
        engine.give(p, cam)
    out["has_occluders"].append(engine.has_occluders())
    out["frames"].append(engine.end(debug))
    # frame 2: tests before any occluder read the grid the first frame left
    engine.begin(color, depth)
    out["has_occluders"].append(engine.has_occluders())
    out["visible"] += [engine.visible(p, cam) for p in props]
    if debug:
        engine.box(props[0], cam, True)
    if use_depth:
        engine.top_rows(cam)
        out["grids"].append(engine.grid())
    for s in [sc.wall, sc.panel, sc.field] + list(props):
        engine.give(s, cam)
    out["frames"].append(engine.end())
    return out


def assert_same(a: dict, b: dict, label: str, grids: bool = True):
    assert a["visible"] == b["visible"], f"{label}: box tests differ"
    assert a["has_occluders"] == b["has_occluders"], f"{label}: has_occluders differs"
    for k, (fa, fb) in enumerate(zip(a["frames"], b["frames"])):
        for i, what in ((0, "colour"), (1, "depth")):
            if fa[i] is None or fb[i] is None:
                assert fa[i] is None and fb[i] is None
                continue
            bad = np.argwhere(np.asarray(fa[i]).view(np.uint32) != np.asarray(fb[i]).view(np.uint32))
            assert len(bad) == 0, f"{label}: frame {k} {what} differs at {len(bad)} pixels, first {bad[:4].tolist()}"
        if fa[2] is not None and fb[2] is not None:
            assert fa[2] == fb[2], f"{label}: frame {k} fragments {fa[2]} != {fb[2]}"
    if grids:
        for k, (ga, gb) in enumerate(zip(a["grids"], b["grids"])):
            if ga is None or gb is None:
                continue
            assert np.array_equal(ga.view(np.uint32), gb.view(np.uint32)), f"{label}: grid {k} differs"
