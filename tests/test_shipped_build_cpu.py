"""How far the reference as shipped (-O2 -march=native: SIMD reciprocals, fused multiply-adds
where the compiler contracts them) lies from the oracle, which equals the exact build and the GPU
bit for bit.  Run here where the reference was built from its sources (skipped elsewhere).

The renderer's arithmetic is a chain of binary32 operations: the shipped build's `rcp` + Newton
steps (simd.h:4045-4068) and contracted products change low bits of depth in many pixels, and where
two triangles' depths are that close the depth test picks the other one, so a few pixels take
another triangle's colour.  The set of pixels drawn (the row intervals are exact integer work)
must be the same.  The test prints the mismatch table and holds the figures to their measured size.
"""
import numpy as np
import pytest

from dfpsr_gb300 import scenes


@pytest.fixture(scope="module")
def shipped(built):
    from oracle import ref
    if not (ref.available("shipped") and ref.available("exact")):
        pytest.skip("the reference was not built from source on this machine")
    return ref


def _mismatch(scene, ref):
    from oracle import port
    sc, sd = ref.RefModel(scene, "shipped").render()
    oc, od, _ = port.render(scene)
    drawn_shipped, drawn_oracle = sd != 0.0, od != 0.0  # depth cleared to 0 = infinitely far
    channels = np.abs(sc.view(np.uint8).astype(np.int32) - oc.view(np.uint8).astype(np.int32)).reshape(sc.shape + (4,))
    lsb = channels.max(axis=2)
    depth_bad = sd.view(np.uint32) != od.view(np.uint32)
    rel = np.abs(sd.astype(np.float64) - od.astype(np.float64)) / np.maximum(np.abs(od.astype(np.float64)), 1e-30)
    return {
        "pixels": int(sc.size),
        "drawn": int(drawn_oracle.sum()),
        "drawn_set_differs": int((drawn_shipped != drawn_oracle).sum()),
        "colour_px": int((lsb > 0).sum()),
        "colour_px_over_1_lsb": int((lsb > 1).sum()),
        "colour_max_lsb": int(lsb.max()),
        "depth_px": int(depth_bad.sum()),
        "depth_max_rel": float(rel[drawn_oracle].max()) if drawn_oracle.any() else 0.0,
        "depth_px_over_1e-6": int((rel[drawn_oracle] > 1e-6).sum()),
    }


CASES = {
    "800x600 random 20k": lambda: scenes.random_triangles(seed=1234),
    "1920x1080 terrain 522k": lambda: scenes.terrain(seed=1234),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_shipped_build_mismatch_report(shipped, name):
    m = _mismatch(CASES[name](), shipped)
    print(f"\nshipped build vs oracle, {name}: " + ", ".join(f"{k} {v}" for k, v in m.items()))
    assert m["drawn_set_differs"] == 0  # coverage is integer work: identical
    # measured here (x86-64, AVX-512): C0 793 colour pixels (34 over 1 LSB), depth max relative
    # 8.7e-5; terrain 75,646 colour pixels (1,781 over 1 LSB), depth max relative 1.2e-2, where far
    # triangles' planes cancel (start + dx*x + dy*y) and a contracted product moves the small sum
    assert m["colour_px_over_1_lsb"] <= 0.002 * m["pixels"]
    assert m["colour_px"] <= 0.05 * m["pixels"]
    assert m["depth_max_rel"] < 0.05
