"""The oracle's restatement of the sprite engine's dense models (DenseModel_create and
renderDenseModel, SDK/SpriteEngine/spriteAPI.cpp:1156-1327) against the reference itself, built
from source here: height, diffuse and normal images bit for bit, in both qualities, every view
direction, over empty and prefilled images and with the model moved around."""
import numpy as np
import pytest

from dfpsr_gb300 import scenes


def _both(sc, high_quality, variant="exact"):
    from oracle import port, ref
    view = port.ortho_view(sc.camera_tilt, sc.pixels_per_tile, sc.view_index)
    tris = port.dense_model(sc.positions, sc.polygons, sc.colors)
    o = port.dense_render(tris, view, sc.height, sc.diffuse, sc.normal, sc.origin, sc.model_to_world, high_quality)
    r = ref.dense_render(sc.positions, sc.polygons, sc.colors, sc.camera_tilt, sc.pixels_per_tile, sc.view_index, sc.height,
                         sc.diffuse, sc.normal, sc.origin, sc.model_to_world, high_quality, variant)
    return o, r


@pytest.mark.parametrize("high_quality", [False, True])
@pytest.mark.parametrize("view_index,prefilled", [(0, False), (3, True), (5, False), (6, True)])
def test_oracle_dense_render_equals_reference(built, high_quality, view_index, prefilled):
    from oracle import ref
    if not ref.available("exact"):
        pytest.skip("the reference was not built from source on this machine")
    sc = scenes.dense_scene(seed=20 + view_index, view_index=view_index, prefilled=prefilled)
    (oh, od, on), (rh, rd, rn) = _both(sc, high_quality)
    assert np.array_equal(oh.view(np.uint32), rh.view(np.uint32)), "height differs"
    assert np.array_equal(od, rd), f"{int((od != rd).sum())} diffuse pixels differ"
    assert np.array_equal(on, rn), f"{int((on != rn).sum())} normal pixels differ"
    assert int((od != sc.diffuse).sum()) > 1000  # the model was drawn


def test_oracle_dense_model_partly_outside(built):
    from oracle import ref
    if not ref.available("exact"):
        pytest.skip("the reference was not built from source on this machine")
    sc = scenes.dense_scene(seed=31, width=160, height=96)
    sc.origin = (10.0, 90.0)  # the torus crosses the left and bottom edges
    (oh, od, on), (rh, rd, rn) = _both(sc, True)
    assert np.array_equal(oh.view(np.uint32), rh.view(np.uint32))
    assert np.array_equal(od, rd) and np.array_equal(on, rn)
