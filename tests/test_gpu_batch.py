"""Batched rendering (dsrg_batch_*): every frame of a batch must equal the same frame drawn alone
through dsrg_model_render / dsrg_renderer_*, which the other GPU tests hold to the oracle; one
frame is also checked against the oracle directly.  Covers mixed resolutions, host and device
images, several tasks per frame given interleaved across frames, repeated renders (the CUDA
graph replay path), every launch shape the autotuner can choose, and the autotuner itself."""
import numpy as np
import pytest

from dfpsr_gb300 import scenes

pytestmark = pytest.mark.gpu


def _frames(seed=11, frames=7, max_triangles=3000):
    res = ((64, 64), (256, 256), (200, 120), (96, 160))
    return scenes.batch_frames(seed=seed, frames=frames, resolutions=res, min_triangles=200, max_triangles=max_triangles,
                               texture_size=64)


def _alone(ctx, model, scene, color=True, depth=True):
    import dfpsr_gb300 as d
    c = np.zeros((scene.height, scene.width), np.uint32) if color else None
    z = np.zeros((scene.height, scene.width), np.float32) if depth else None
    ctx.render(model, model.camera, c, z)
    return c, z


def _same(a, b):
    if a is None or b is None:
        return a is None and b is None
    return np.array_equal(np.asarray(a).view(np.uint32), np.asarray(b).view(np.uint32))


def test_batch_frames_equal_frames_rendered_alone(ctx):
    import torch
    import dfpsr_gb300 as d
    frame_scenes = _frames()
    models = [d.Model(ctx, s) for s in frame_scenes]
    expected = [_alone(ctx, m, s) for m, s in zip(models, frame_scenes)]
    batch = d.Batch(ctx)
    images = []
    for i, (m, s) in enumerate(zip(models, frame_scenes)):
        if i % 3 == 0:  # pageable host images (staged through device buffers)
            c = np.zeros((s.height, s.width), np.uint32)
            z = np.zeros((s.height, s.width), np.float32)
        elif i % 3 == 1:  # page-locked host images with padded rows (drawn in place)
            c = torch.zeros((s.height, s.width + 5), dtype=torch.int32).pin_memory().numpy()[:, : s.width]
            z = torch.zeros((s.height, s.width + 3), dtype=torch.float32).pin_memory().numpy()[:, : s.width]
        else:  # device images
            c = torch.zeros((s.height, s.width), dtype=torch.int32, device="cuda")
            z = torch.zeros((s.height, s.width), dtype=torch.float32, device="cuda")
        images.append((c, z))
        assert batch.add_frame(c, z) == i
        batch.give_task(i, m)
    for round_ in range(3):  # the second render captures each phase's graph, the third replays it
        for c, z in images:
            if isinstance(c, np.ndarray):
                c[:] = 0
                z[:] = 0
            else:
                c.zero_()
                z.zero_()
        batch.render()
        torch.cuda.synchronize()
        for i, ((c, z), (ec, ez)) in enumerate(zip(images, expected)):
            got_c = c if isinstance(c, np.ndarray) else c.cpu().numpy()
            got_z = z if isinstance(z, np.ndarray) else z.cpu().numpy()
            assert _same(got_c, ec), f"round {round_} frame {i}: colour differs from the frame rendered alone"
            assert _same(got_z, ez), f"round {round_} frame {i}: depth differs from the frame rendered alone"
    batch.destroy()


def test_batch_frame_matches_oracle(ctx):
    import dfpsr_gb300 as d
    from oracle import port
    scene = _frames(seed=12, frames=1, max_triangles=1500)[0]
    model = d.Model(ctx, scene)
    batch = d.Batch(ctx)
    c = np.zeros((scene.height, scene.width), np.uint32)
    z = np.zeros((scene.height, scene.width), np.float32)
    batch.add_frame(c, z)
    batch.give_task(0, model)
    batch.render()
    rc, rd, _ = port.render(scene)
    assert np.array_equal(c, rc)
    assert np.array_equal(z.view(np.uint32), rd.view(np.uint32))


def test_batch_interleaved_tasks_keep_each_frames_submission_order(ctx):
    """Two frames, three overlapping models each, tasks given alternately between the frames:
    each frame must equal renderer_begin / give_task x3 / end on that frame alone."""
    import dfpsr_gb300 as d
    parts = [scenes.random_triangles(seed=300 + k, triangles=400, width=160, height=128, texture_size=32) for k in range(3)]
    models = [d.Model(ctx, p) for p in parts]
    cam_a = models[0].camera
    cam_b = d.camera_struct(parts[0])
    loc = scenes.camera_location((0.3, 0.1, -2.8), (-0.1, 0.0, 1.0))
    for i in range(12):
        cam_b.location[i] = float(loc[i])
    expected = []
    for cam in (cam_a, cam_b):
        r = d.Renderer(ctx)
        c = np.zeros((128, 160), np.uint32)
        z = np.zeros((128, 160), np.float32)
        r.begin(c, z)
        for m in models:
            r.give_task(m, cam)
        r.end()
        expected.append((c, z))
    batch = d.Batch(ctx)
    imgs = [(np.zeros((128, 160), np.uint32), np.zeros((128, 160), np.float32)) for _ in range(2)]
    for c, z in imgs:
        batch.add_frame(c, z)
    for m in models:
        batch.give_task(0, m, cam_a)
        batch.give_task(1, m, cam_b)
    batch.render()
    for (c, z), (ec, ez) in zip(imgs, expected):
        assert _same(c, ec) and _same(z, ez)


@pytest.mark.parametrize("threads,per_sm,small,resolve", [(256, 4, (8, 16), 1), (256, 1, (0, 0), 2), (128, 8, (16, 32), 2),
                                                           (128, 2, (4, 8), 1), (64, 16, (8, 16), 2), (64, 3, (0, 0), 1),
                                                           (128, 8, (8, 16), 0)])
def test_every_launch_shape_gives_the_same_frames(ctx, threads, per_sm, small, resolve):
    import dfpsr_gb300 as d
    frame_scenes = _frames(seed=13, frames=4, max_triangles=2500)
    models = [d.Model(ctx, s) for s in frame_scenes]
    expected = [_alone(ctx, m, s) for m, s in zip(models, frame_scenes)]
    before = ctx.tuning()
    try:
        ctx.set_tuning(threads_per_tile=threads, ctas_per_sm=per_sm, small_rows=small[0], small_width=small[1], resolve=resolve)
        batch = d.Batch(ctx)
        imgs = []
        for i, (m, s) in enumerate(zip(models, frame_scenes)):
            imgs.append((np.zeros((s.height, s.width), np.uint32), np.zeros((s.height, s.width), np.float32)))
            batch.add_frame(*imgs[-1])
            batch.give_task(i, m)
        batch.render()
        for (c, z), (ec, ez) in zip(imgs, expected):
            assert _same(c, ec) and _same(z, ez)
        # the plain path with the same shape
        for m, s, (ec, ez) in zip(models, frame_scenes, expected):
            c, z = _alone(ctx, m, s)
            assert _same(c, ec) and _same(z, ez)
    finally:
        ctx.set_tuning(**{k: v for k, v in before.items()})


def test_autotune_picks_a_valid_shape_and_keeps_results(ctx):
    import dfpsr_gb300 as d
    frame_scenes = _frames(seed=14, frames=5, max_triangles=2000)
    models = [d.Model(ctx, s) for s in frame_scenes]
    expected = [_alone(ctx, m, s) for m, s in zip(models, frame_scenes)]
    before = ctx.tuning()
    try:
        batch = d.Batch(ctx)
        imgs = []
        for i, (m, s) in enumerate(zip(models, frame_scenes)):
            imgs.append((np.zeros((s.height, s.width), np.uint32), np.zeros((s.height, s.width), np.float32)))
            batch.add_frame(*imgs[-1])
            batch.give_task(i, m)
        best = batch.autotune(rounds=1)
        assert best["threads_per_tile"] in (64, 128, 256)
        assert best["resolve"] in (0, 1, 2)
        assert 1 <= best["ctas_per_sm"] <= 1024 // best["threads_per_tile"]
        assert ctx.tuning() == best
        for c, z in imgs:
            c[:] = 0
            z[:] = 0
        batch.render()
        for (c, z), (ec, ez) in zip(imgs, expected):
            assert _same(c, ec) and _same(z, ez)
    finally:
        ctx.set_tuning(**{k: v for k, v in before.items()})


def test_depth_only_frame_and_errors(ctx):
    import dfpsr_gb300 as d
    scene = _frames(seed=15, frames=1, max_triangles=800)[0]
    model = d.Model(ctx, scene)
    _, ez = _alone(ctx, model, scene, color=False)
    batch = d.Batch(ctx)
    z = np.zeros((scene.height, scene.width), np.float32)
    batch.add_frame(None, z)
    batch.give_task(0, model)
    batch.render()
    assert _same(z, ez)
    with pytest.raises(d.DsrgError) as e:
        batch.give_task(5, model)
    assert e.value.status == 1
    with pytest.raises(d.DsrgError):
        batch.add_frame(None, None)
    with pytest.raises(d.DsrgError):
        ctx.set_tuning(threads_per_tile=96)
    with pytest.raises(d.DsrgError):
        ctx.set_tuning(threads_per_tile=256, ctas_per_sm=5)
    with pytest.raises(d.DsrgError):
        ctx.set_tuning(resolve=3)


def test_benchmarked_batch_frames_match_oracle(ctx):
    """Frames of the benchmarked mixed-size batch itself (scenes.batch_frames(seed=4321): 256 frames,
    resolutions 64x64 to 1024x768, 1k-200k random triangles each): the 12 frames with the most
    triangles at 1024x768 and 640x480 and two of each smaller resolution, rendered together in one
    batch after the autotuner, each compared bit for bit with the oracle (12 row bands on all
    host cores, which equals the single-band oracle)."""
    import os
    import dfpsr_gb300 as d
    from oracle import port
    frames = scenes.batch_frames(seed=4321)
    by_size = {}
    for i, s in enumerate(frames):
        by_size.setdefault((s.width, s.height), []).append(i)
    chosen = []
    for size, count in (((1024, 768), 4), ((640, 480), 4), ((256, 256), 2), ((64, 64), 2)):
        chosen += sorted(by_size[size], key=lambda i: -frames[i].triangle_count)[:count]
    assert any(frames[i].width == 1024 and frames[i].triangle_count > 100_000 for i in chosen)
    before = ctx.tuning()
    try:
        batch = d.Batch(ctx)
        imgs = []
        for k, i in enumerate(chosen):
            s = frames[i]
            m = d.Model(ctx, s)
            imgs.append((np.zeros((s.height, s.width), np.uint32), np.zeros((s.height, s.width), np.float32)))
            batch.add_frame(*imgs[-1])
            batch.give_task(k, m)
        batch.autotune(rounds=1)
        for c, z in imgs:
            c[:] = 0
            z[:] = 0
        batch.render()
        threads = os.cpu_count() or 1
        for (c, z), i in zip(imgs, chosen):
            s = frames[i]
            rc, rd, _ = port.render(s, bands=12, threads=threads)
            label = f"frame {i} ({s.width}x{s.height}, {s.triangle_count} triangles)"
            assert np.array_equal(c, rc), f"{label}: {int((c != rc).sum())} colour pixels differ"
            assert np.array_equal(z.view(np.uint32), rd.view(np.uint32)), f"{label}: depth differs"
        batch.destroy()
    finally:
        ctx.set_tuning(**{k: v for k, v in before.items()})


def test_depth_only_batch_with_more_tiles_than_one_launch_covers(ctx):
    """A depth-only batch (the shadow-map form) of 40 frames of 2048 x 2048: 655,360 tiles, more than
    one pass of the totals launch's grid lists, so the listing of the tiles that have entries must
    stride over them.  Every frame against the oracle's model_renderDepth, bit for bit."""
    import torch
    import dfpsr_gb300 as d
    from oracle import port
    batch = d.Batch(ctx)
    batch.set_depth_only(True)
    scenes_, images, models = [], [], []
    for k in range(40):
        s = scenes.random_triangles(seed=700 + k, triangles=60, width=2048, height=2048, texture_size=0)
        scenes_.append(s)
        m = d.Model(ctx, s)
        models.append(m)
        images.append(torch.zeros((2048, 2048), dtype=torch.float32, device="cuda"))
        batch.add_frame(None, images[-1])
        batch.give_task(k, m)
    batch.render()
    for k in (0, 13, 26, 39):  # frames from the start, the middle and the end of the tile range
        want, _ = port.render_depth(scenes_[k])
        assert np.array_equal(images[k].cpu().numpy().view(np.uint32), want.view(np.uint32)), f"frame {k}"
        assert (want != 0).sum() > 1000
    batch.destroy()
    for m in models:
        m.destroy()


def test_batch_with_a_tuning_of_its_own(ctx):
    """dsrg_batch_set_tuning: the batch renders with its own configuration, the context's is left
    as it was (also by the autotuner, which then keeps its choice for the batch), the images are
    those of the frames drawn one by one, and a configuration out of range is refused."""
    import dfpsr_gb300 as d
    frame_scenes = _frames(seed=15, frames=4, max_triangles=2000)
    models = [d.Model(ctx, s) for s in frame_scenes]
    expected = [_alone(ctx, m, s) for m, s in zip(models, frame_scenes)]
    before = ctx.tuning()
    try:
        batch = d.Batch(ctx)
        imgs = []
        for i, (m, s) in enumerate(zip(models, frame_scenes)):
            imgs.append((np.zeros((s.height, s.width), np.uint32), np.zeros((s.height, s.width), np.float32)))
            batch.add_frame(*imgs[-1])
            batch.give_task(i, m)
        own = dict(before, threads_per_tile=64, ctas_per_sm=16, resolve=2)
        batch.set_tuning(own)
        batch.render()
        assert ctx.tuning() == before
        for (c, z), (ec, ez) in zip(imgs, expected):
            assert _same(c, ec) and _same(z, ez)
        best = batch.autotune(rounds=1)
        assert ctx.tuning() == before
        assert best["threads_per_tile"] in (64, 128, 256)
        for c, z in imgs:
            c[:] = 0
            z[:] = 0
        batch.render()
        assert ctx.tuning() == before
        for (c, z), (ec, ez) in zip(imgs, expected):
            assert _same(c, ec) and _same(z, ez)
        with pytest.raises(d.DsrgError, match="threadsPerTile"):
            batch.set_tuning(dict(before, threads_per_tile=96))
        batch.set_tuning(None)
        batch.render()
        assert ctx.tuning() == before
        batch.destroy()
    finally:
        ctx.set_tuning(**{k: v for k, v in before.items()})
        for m in models:
            m.destroy()
