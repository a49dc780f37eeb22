"""Edge cases of dsrg_model_render against the oracle, bit-exact: a model without polygons,
triangles that never reach the target (behind the camera, beside the frustum), degenerate
triangles (repeated and collinear corners), targets a few pixels wide, and a fresh context whose
first frames outgrow every learned buffer capacity (the frame is redone internally)."""
import dataclasses

import numpy as np
import pytest

from dfpsr_gb300 import scenes

pytestmark = pytest.mark.gpu


def _render_both(ctx, scene, color=None, depth=None):
    import dfpsr_gb300 as d
    from oracle import port
    ctx.set_counting(True)
    try:
        c, z = d.render_scene(ctx, scene, None if color is None else color.copy(), None if depth is None else depth.copy())
        stats = ctx.stats()
    finally:
        ctx.set_counting(False)
    rc, rz, info = port.render(scene, color, depth)
    return (c, z, stats["fragments"]), (rc, rz, info["fragments"])


def _assert_same(got, expect, label):
    (c, z, f), (rc, rz, rf) = got, expect
    assert np.array_equal(c, rc), f"{label}: {int((c != rc).sum())} colour pixels differ"
    assert np.array_equal(z.view(np.uint32), rz.view(np.uint32)), f"{label}: depth differs"
    assert f == rf, label


def _prefilled(seed, h, w):
    rng = np.random.default_rng(seed)
    return (rng.integers(0, 2**32, size=(h, w), dtype=np.uint64).astype(np.uint32),
            rng.uniform(0.0, 0.1, size=(h, w)).astype(np.float32))


def test_model_without_polygons_leaves_targets(ctx):
    s = scenes.random_triangles(seed=61, triangles=10, width=64, height=48)
    empty = dataclasses.replace(s, poly_indices=np.zeros((0, 4), np.int32), tex_coords=np.zeros((0, 4, 4), np.float32),
                                colors=np.zeros((0, 4, 4), np.float32))
    color, depth = _prefilled(1, 48, 64)
    got, expect = _render_both(ctx, empty, color, depth)
    _assert_same(got, expect, "empty")
    assert np.array_equal(got[0], color) and got[2] == 0


@pytest.mark.parametrize("where", ["behind", "beside"])
def test_triangles_that_miss_the_target(ctx, where):
    s = scenes.random_triangles(seed=62, triangles=400, width=128, height=96)
    pos = s.positions.copy()
    if where == "behind":
        pos[:, 2] -= 6.0  # the camera sits at z = -3 looking toward +z
    else:
        pos[:, 0] += 40.0  # far to the right of the frustum
    color, depth = _prefilled(2, 96, 128)
    got, expect = _render_both(ctx, dataclasses.replace(s, positions=pos), color, depth)
    _assert_same(got, expect, where)
    assert np.array_equal(got[0], color) and got[2] == 0


def test_degenerate_triangles(ctx):
    s = scenes.random_triangles(seed=63, triangles=900, width=160, height=120)
    pos = s.positions.copy()
    poly = s.poly_indices.copy()
    rng = np.random.default_rng(5)
    repeated = rng.choice(len(poly), 150, replace=False)
    poly[repeated, 1] = poly[repeated, 0]                      # two corners the same
    collinear = rng.choice(np.setdiff1d(np.arange(len(poly)), repeated), 150, replace=False)
    a, b = pos[poly[collinear, 0]], pos[poly[collinear, 1]]
    pos[poly[collinear, 2]] = (a + b) * np.float32(0.5)        # third corner on the first edge
    tiny = rng.choice(np.setdiff1d(np.arange(len(poly)), np.concatenate([repeated, collinear])), 150, replace=False)
    pos[poly[tiny, 1]] = pos[poly[tiny, 0]] + np.float32(1e-4)  # sub-pixel slivers
    pos[poly[tiny, 2]] = pos[poly[tiny, 0]] + np.float32(2e-4)
    got, expect = _render_both(ctx, dataclasses.replace(s, positions=pos, poly_indices=poly))
    _assert_same(got, expect, "degenerate")


@pytest.mark.parametrize("size", [(1, 2), (2, 2), (3, 4), (17, 2), (5, 34)])
def test_targets_a_few_pixels_wide(ctx, size):
    w, h = size
    s = scenes.random_triangles(seed=64, triangles=300, width=w, height=h, texture_size=16)
    got, expect = _render_both(ctx, s)
    _assert_same(got, expect, f"{w}x{h}")


def test_fresh_context_outgrows_its_buffers(built):
    """The first frame of a context sizes records, rows and tile lists from its triangle count;
    large triangles need far more rows and list entries, so the frame is redone with the totals
    it reported.  Every frame must still equal the oracle, also a small one afterwards."""
    import dfpsr_gb300 as d
    fresh = d.Context(0)
    try:
        small = scenes.random_triangles(seed=65, triangles=200, width=96, height=64)
        big = scenes.random_triangles(seed=66, triangles=3000, width=640, height=480)
        for label, scene in (("small", small), ("big", big), ("small again", small)):
            got, expect = _render_both(fresh, scene)
            _assert_same(got, expect, label)
    finally:
        fresh.close()
