"""The FP64 oracle of the differentiable renderer on its own (no GPU): on a synthetic
visibility buffer, its analytic gradients equal central finite differences of its loss."""
import numpy as np

from dfpsr_gb300 import scenes
from oracle import diff64


def synthetic_visibility(problem, rng, pixels=3000):
    slots = diff64.fan_triangles(problem.mesh.poly_indices)
    vis = np.zeros((pixels, 3), np.uint32)
    vis[:, 0] = rng.integers(0, len(slots), size=pixels)
    b = rng.uniform(0, 1, size=pixels).astype(np.float32)
    c = (rng.uniform(0, 1, size=pixels) * (1 - b)).astype(np.float32)
    vis[:, 1] = b.view(np.uint32)
    vis[:, 2] = c.view(np.uint32)
    vis[rng.uniform(size=pixels) < 0.2, 0] = diff64.NO_TRIANGLE
    return vis


def test_fp64_gradients_equal_finite_differences():
    problem = scenes.diff_problem(seed=3, views=1, size=32, texture_size=16, major=12, minor=8)
    rng = np.random.default_rng(1)
    vis = synthetic_visibility(problem, rng)
    shading = diff64.Shading(problem.mesh, vis, problem.texture.shape)
    targets = rng.uniform(0, 1, size=(len(vis), 4))
    out, _ = shading.forward(problem.texture, problem.vertex_colors, problem.light, problem.ambient)
    g = shading.gradients(problem.texture, problem.vertex_colors, problem.light, problem.ambient, diff64.l2_grad(out, targets))
    base = [problem.texture.astype(np.float64), problem.vertex_colors.astype(np.float64), problem.light.astype(np.float64)]
    h = 1e-5
    for gi in range(3):
        flat = g[gi].reshape(-1)
        touched = np.nonzero(flat)[0]
        for idx in rng.choice(touched, size=min(6, len(touched)), replace=False):
            plus = [b.copy() for b in base]
            minus = [b.copy() for b in base]
            plus[gi].reshape(-1)[idx] += h
            minus[gi].reshape(-1)[idx] -= h
            fd = (shading.loss(*plus, problem.ambient, targets) - shading.loss(*minus, problem.ambient, targets)) / (2 * h)
            assert abs(fd - flat[idx]) <= 1e-4 * abs(fd) + 1e-12, (gi, idx, fd, flat[idx])


def test_uncovered_pixels_are_black_and_taps_wrap():
    problem = scenes.diff_problem(seed=4, views=1, size=32, texture_size=16, major=12, minor=8)
    rng = np.random.default_rng(2)
    vis = synthetic_visibility(problem, rng, pixels=500)
    shading = diff64.Shading(problem.mesh, vis, problem.texture.shape)
    out, _ = shading.forward(problem.texture, problem.vertex_colors, problem.light, problem.ambient)
    assert np.all(out[vis[:, 0] == diff64.NO_TRIANGLE] == 0)
    assert shading.taps.min() >= 0 and shading.taps.max() < 16 * 16
    np.testing.assert_allclose(shading.tap_weights.sum(axis=1), 1.0)
