"""Failure paths made on the host: the library's device allocations go through one wrapper, and
dsrg_debug_fail_allocation makes the k-th of them fail as an exhausted GPU would.  Every call that
meets the failure must return DSRG_ERROR_OUT_OF_MEMORY with a message, and the context must keep
working: the same frame, drawn again, equals the oracle.  Nothing here faults the GPU."""
import numpy as np
import pytest

from dfpsr_gb300 import scenes

pytestmark = pytest.mark.gpu

OUT_OF_MEMORY = 3


@pytest.fixture
def no_injection():
    import dfpsr_gb300 as d
    yield d
    d.lib().dsrg_debug_fail_allocation(-1)


def test_every_allocation_of_a_first_frame_can_fail_and_be_recovered(built, no_injection):
    d = no_injection
    from oracle import port
    scene = scenes.random_triangles(seed=81, triangles=1500, width=256, height=192, texture_size=64)
    rc, rd, _ = port.render(scene)
    failures = 0
    for k in range(64):
        ctx = d.Context(0)
        try:
            d.lib().dsrg_debug_fail_allocation(k)
            failed = False
            try:
                model = d.Model(ctx, scene)  # texture pyramid and model arrays
                color, depth = d.render_scene(ctx, scene, model=model)  # the context's frame buffers grow here
            except d.DsrgError as e:
                assert e.status == OUT_OF_MEMORY, str(e)
                assert e.message, "an error without a message"
                failed = True
                failures += 1
            d.lib().dsrg_debug_fail_allocation(-1)
            # the same context draws the frame correctly afterwards
            model = d.Model(ctx, scene)
            color, depth = d.render_scene(ctx, scene, model=model)
            assert np.array_equal(color, rc), f"after a failure at allocation {k}"
            assert np.array_equal(depth.view(np.uint32), rd.view(np.uint32)), f"after a failure at allocation {k}"
        finally:
            ctx.close()
        if not failed:
            break  # k is past the last allocation the first frame makes
    assert failures >= 5  # the model, its texture and several frame buffers were each refused once
    assert not failed


def test_failed_batch_and_texture_allocations_leave_the_context_usable(ctx, no_injection):
    d = no_injection
    from oracle import port
    scenes_ = [scenes.random_triangles(seed=90 + i, triangles=800, width=96 + 32 * i, height=80, texture_size=32) for i in range(3)]
    models = [d.Model(ctx, s) for s in scenes_]
    # a texture whose pyramid cannot be allocated
    d.lib().dsrg_debug_fail_allocation(0)
    with pytest.raises(d.DsrgError) as e:
        d.Texture(ctx, np.zeros((64, 64), np.uint32), 4)
    assert e.value.status == OUT_OF_MEMORY
    d.lib().dsrg_debug_fail_allocation(-1)
    # a batch larger than anything the context drew so far, with its first buffer growth refused
    big = scenes.random_triangles(seed=99, triangles=60000, width=1024, height=768, texture_size=32)
    big_model = d.Model(ctx, big)
    batch = d.Batch(ctx)
    images = []
    for i, (s, m) in enumerate(zip(scenes_ + [big], models + [big_model])):
        images.append((np.zeros((s.height, s.width), np.uint32), np.zeros((s.height, s.width), np.float32)))
        batch.add_frame(*images[-1])
        batch.give_task(i, m)
    d.lib().dsrg_debug_fail_allocation(0)
    with pytest.raises(d.DsrgError) as e:
        batch.render()
    assert e.value.status == OUT_OF_MEMORY
    d.lib().dsrg_debug_fail_allocation(-1)
    for c, z in images:
        c[:] = 0
        z[:] = 0
    batch.render()
    import os
    for (c, z), s in zip(images, scenes_ + [big]):
        rc, rd, _ = port.render(s, bands=12, threads=os.cpu_count() or 1)
        assert np.array_equal(c, rc) and np.array_equal(z.view(np.uint32), rd.view(np.uint32))
    batch.destroy()
