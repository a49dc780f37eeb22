"""Host parts of the light passes, against the reference build (no GPU): the library's OrthoView and
shadow-cube camera locations equal the reference's OrthoSystem and PointLight matrices bit for bit."""
import numpy as np
import pytest

from oracle import port, ref


@pytest.mark.parametrize("tilt,ppt", [(-1.0, 64), (-0.5, 32), (-0.7, 100), (-2.0, 48)])
def test_ortho_views_match(built, tilt, ppt):
    import dfpsr_gb300 as d
    for index in range(8):
        m, i = d.ortho_view(tilt, ppt, index).arrays()
        pm, pi = port.ortho_view(tilt, ppt, index).arrays()
        assert np.array_equal(m.view(np.uint32), pm.view(np.uint32)) and np.array_equal(i, pi)
        if ref.available():
            rm, ri = ref.ortho_view(tilt, ppt, index)
            assert np.array_equal(m.view(np.uint32), rm.view(np.uint32)) and np.array_equal(i, ri)


def test_shadow_sides_match(built):
    import dfpsr_gb300 as d
    for index in (0, 3, 6):
        n = np.ctypeslib.as_array(d.ortho_view(-0.8, 64, index).normalToWorld).copy()
        for side in range(6):
            loc = d.shadow_side_location(n, side)
            assert np.array_equal(loc.view(np.uint32), port.shadow_side(n, side).view(np.uint32))
            if ref.available():
                assert np.array_equal(loc.view(np.uint32), ref.shadow_side(n, side).view(np.uint32))


def test_oracle_light_pass_equals_the_reference_frame(built):
    """The oracle's whole deferred-light frame (oracle/light_pass.py: clears, draw_higher of every
    sprite, six model_renderDepth faces per shadowed light, setDirectedLight, addPointLight per
    light with the reference's thread bands, blendLight) equals the same frame made by the
    reference's own functions (refh_light_frame, exact build), image by image, bit for bit."""
    if not ref.available():
        pytest.skip("the reference was not built from source on this machine")
    from dfpsr_gb300 import scenes
    from oracle import light_pass
    view = port.ortho_view(-0.7, 64, 0)
    m = np.concatenate([np.ctypeslib.as_array(view.normalToWorld), np.ctypeslib.as_array(view.screenDepthToLightSpace)])
    scene = scenes.light_scene(seed=3, width=320, height=300, sprites=150, sprite_types=6, lights=4, radius_px=(60, 150),
                               caster_triangles=300, cube_resolution=64, light_space=(m[9:18], m[0:9]))
    threads = ref.thread_count("exact")
    out, light, height, diffuse, normal, cubes = light_pass.run(scene, threads, workers=2)
    _, ref_out, ref_light, ref_height, ref_cubes = ref.light_frame(scene, 1, variant="exact")
    assert np.array_equal(height.view(np.uint32), ref_height.view(np.uint32))
    for k, (a, b) in enumerate(zip(cubes, ref_cubes)):
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), f"shadow cube {k}"
    assert np.array_equal(light, ref_light)
    assert np.array_equal(out, ref_out)
    assert (out != 0).mean() > 0.3
