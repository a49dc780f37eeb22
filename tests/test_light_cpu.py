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
