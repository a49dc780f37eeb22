"""Frames whose tasks differ in kind, against the oracle, bit for bit: alpha-filtered and solid
models, perspective and orthogonal cameras, in any order within one frame.  Each triangle tests
depth with its own projection's comparison (fillerTemplates.h:108-152) and alpha-filtered ones
blend in submission order (fillerTemplates.h:387-441), so a frame is drawn as consecutive runs of
tasks of one kind.  Covers the renderer (renderer_begin / giveTask / end) and the batch, whose
frames may each hold a different sequence of runs."""
import dataclasses

import numpy as np
import pytest

from dfpsr_gb300 import scenes

pytestmark = pytest.mark.gpu


def _task(seed, w, h, perspective=True, alpha=False, shift=0.0, triangles=700):
    s = scenes.random_triangles(seed=seed, triangles=triangles, width=w, height=h, texture_size=32)
    if not perspective:
        s.perspective = False
        s.slope = 1.3
    if alpha:
        s = dataclasses.replace(s, filter=1)
    s.model_to_world = np.array([shift, -0.5 * shift, 2.0 * shift, 1, 0, 0, 0, 1, 0, 0, 0, 1], np.float32)
    return s


def _mixed(w, h, seed=140):
    kinds = [(True, False), (False, False), (True, True), (False, True), (True, False)]
    return [_task(seed + i, w, h, p, a, 0.1 * i) for i, (p, a) in enumerate(kinds)]


def _oracle_frame(tasks, color0, depth0):
    from oracle import port
    o = port.OracleRenderer()
    o.begin(color0, depth0)
    pms = [port.PreparedModel(s) for s in tasks]
    for s, pm in zip(tasks, pms):
        o.give_task(pm, s.model_to_world, pm.cam)
    c, d, _ = o.end()
    return c, d


def _prefilled(h, w, seed=3):
    rng = np.random.default_rng(seed)
    return (rng.integers(0, 2**32, size=(h, w), dtype=np.uint64).astype(np.uint32),
            rng.uniform(0.0, 0.3, size=(h, w)).astype(np.float32))


@pytest.mark.parametrize("use_depth", [True, False])
def test_renderer_frame_mixing_projections_and_filters(ctx, use_depth):
    import dfpsr_gb300 as d
    tasks = _mixed(211, 143)
    color0, depth0 = _prefilled(143, 211)
    if not use_depth:
        depth0 = None
    rc, rd = _oracle_frame(tasks, color0, depth0)
    models = [d.Model(ctx, s) for s in tasks]
    color = color0.copy()
    depth = None if depth0 is None else depth0.copy()
    r = ctx.renderer()
    r.begin(color, depth)
    for m, s in zip(models, tasks):
        r.give_task(m, m.camera, s.model_to_world)
    r.end()
    assert np.array_equal(color, rc), f"{int((color != rc).sum())} colour pixels differ"
    if use_depth:
        assert np.array_equal(depth.view(np.uint32), rd.view(np.uint32))


def test_batch_frames_with_alpha_and_mixed_projections(ctx):
    """Five frames in one batch: the mixed sequence above, alpha-filtered models only, solid
    perspective only, orthogonal then perspective, and an alpha-filtered model on a frame without a
    colour image (drawn like a solid one); each equals the oracle's frame."""
    import dfpsr_gb300 as d
    frames = [
        _mixed(211, 143),
        [_task(160, 160, 120, alpha=True), _task(161, 160, 120, alpha=True, shift=0.2)],
        [_task(162, 96, 64)],
        [_task(163, 128, 97, perspective=False), _task(164, 128, 97, shift=0.3)],
        [_task(165, 100, 80, alpha=True)],
    ]
    has_color = [True, True, True, True, False]
    batch = d.Batch(ctx)
    images, expected, keep = [], [], []
    for k, (tasks, colored) in enumerate(zip(frames, has_color)):
        h, w = tasks[0].height, tasks[0].width
        color0, depth0 = _prefilled(h, w, seed=10 + k)
        if not colored:
            color0 = None
        expected.append(_oracle_frame(tasks, color0, depth0))
        c = None if color0 is None else color0.copy()
        z = depth0.copy()
        images.append((c, z))
        assert batch.add_frame(c, z) == k
    # tasks given interleaved across frames: each frame keeps its own order
    for i in range(max(len(t) for t in frames)):
        for k, tasks in enumerate(frames):
            if i < len(tasks):
                m = d.Model(ctx, tasks[i])
                keep.append(m)
                batch.give_task(k, m, m.camera, tasks[i].model_to_world)
    for round_ in range(2):  # the second render replays the phases' graphs
        batch.render()
        for k, ((c, z), (rc, rd)) in enumerate(zip(images, expected)):
            if c is not None:
                assert np.array_equal(c, rc), f"round {round_} frame {k}: {int((c != rc).sum())} colour pixels differ"
            assert np.array_equal(z.view(np.uint32), rd.view(np.uint32)), f"round {round_} frame {k}: depth differs"
        # reset the targets for the replay
        for k, (tasks, colored) in enumerate(zip(frames, has_color)):
            h, w = tasks[0].height, tasks[0].width
            color0, depth0 = _prefilled(h, w, seed=10 + k)
            c, z = images[k]
            if c is not None:
                c[:] = color0
            z[:] = depth0
    batch.destroy()
