"""Differentiable rendering (dsrg_diff_*) against the FP64 host oracle (oracle/diff64.py).

- coverage and visibility equal dsrg_model_render's depth-tested coverage of the same views;
- the float forward pass equals the FP64 re-shade at the GPU's visibility (relative 1e-5);
- the adjoint (atomic and deterministic modes) equals the FP64 analytic gradient within a
  relative error of 1e-3 (the bar of the benchmark), and the FP64 gradient equals central
  finite differences of the FP64 loss;
- the deterministic mode is bit-identical from run to run;
- with the light factor held at 1, the forward pass reproduces the reference's RgbaMultiply
  colours before the U8 pack (within the 8-bit texel mixing and truncation of the reference).
"""
import numpy as np
import pytest

from dfpsr_gb300 import scenes

pytestmark = pytest.mark.gpu

GRAD_TOLERANCE = 1e-3


def small_problem(seed=5):
    return scenes.diff_problem(seed=seed, views=4, size=96, texture_size=64, major=60, minor=24)


def run_forward(renderer, cameras, problem, params):
    import torch
    views, h, w = len(cameras), problem.height, problem.width
    images = torch.empty((views, h, w, 4), dtype=torch.float32, device="cuda")
    vis = torch.empty((views, h, w, 3), dtype=torch.int32, device="cuda")
    renderer.forward(cameras, problem.mesh.model_to_world, params["texture"], params["vertex_colors"], params["light"],
                     images, vis)
    return images, vis


def gpu_adjoint(renderer, problem, params, vis, grad, deterministic):
    import torch
    g = {k: torch.empty_like(v) for k, v in params.items()}
    views, h, w = vis.shape[0], vis.shape[1], vis.shape[2]
    renderer.adjoint(views, w, h, problem.mesh.model_to_world, params["texture"], params["vertex_colors"], params["light"],
                     vis, grad, g["texture"], g["vertex_colors"], g["light"], deterministic)
    return {k: v.cpu().numpy() for k, v in g.items()}


def test_visibility_matches_model_render_coverage(ctx):
    import torch
    import dfpsr_gb300 as d
    from diff_harness import make_renderer
    problem = small_problem()
    model, renderer, cameras, params = make_renderer(ctx, problem)
    images, vis = run_forward(renderer, cameras, problem, params)
    tri = vis[..., 0].cpu().numpy().view(np.uint32)
    for v, cam in enumerate(cameras):
        depth = np.zeros((problem.height, problem.width), np.float32)
        ctx.render(model, cam, None, depth)
        assert np.array_equal(depth > 0, tri[v] != 0xFFFFFFFF), f"view {v}"
    assert (tri != 0xFFFFFFFF).sum() > 1000
    assert torch.all(images[torch.from_numpy(tri == 0xFFFFFFFF).to(images.device)] == 0)


def test_forward_equals_fp64_reshade(ctx):
    from diff_harness import make_renderer
    from oracle import diff64
    problem = small_problem()
    _, renderer, cameras, params = make_renderer(ctx, problem)
    images, vis = run_forward(renderer, cameras, problem, params)
    shading = diff64.Shading(problem.mesh, vis.cpu().numpy().view(np.uint32), problem.texture.shape)
    out64, _ = shading.forward(problem.texture, problem.vertex_colors, problem.light, problem.ambient)
    assert diff64.relative_error(images.cpu().numpy().reshape(-1, 4), out64) < 1e-5


@pytest.mark.parametrize("deterministic", [False, True])
def test_adjoint_equals_fp64_gradient(ctx, deterministic):
    import torch
    from diff_harness import make_renderer
    from oracle import diff64
    problem = small_problem()
    _, renderer, cameras, params = make_renderer(ctx, problem)
    images, vis = run_forward(renderer, cameras, problem, params)
    target_renderer_params = {"texture": torch.tensor(problem.target_texture, device="cuda"),
                              "vertex_colors": torch.tensor(problem.target_vertex_colors, device="cuda"),
                              "light": torch.tensor(problem.target_light, device="cuda")}
    targets, _ = run_forward(renderer, cameras, problem, target_renderer_params)
    grad = torch.empty_like(images)
    loss = torch.empty(1, device="cuda")
    renderer.l2_loss(images, targets, grad, loss)
    shading = diff64.Shading(problem.mesh, vis.cpu().numpy().view(np.uint32), problem.texture.shape)
    assert abs(float(loss.item()) - shading.loss(problem.texture, problem.vertex_colors, problem.light, problem.ambient,
                                                 targets.cpu().numpy())) < 1e-5
    g64 = shading.gradients(problem.texture, problem.vertex_colors, problem.light, problem.ambient,
                            diff64.l2_grad(images.cpu().numpy(), targets.cpu().numpy()))
    got = gpu_adjoint(renderer, problem, params, vis, grad, deterministic)
    for name, want in zip(("texture", "vertex_colors", "light"), g64):
        err = diff64.relative_error(got[name], want)
        assert err < GRAD_TOLERANCE, f"{name}: relative error {err}"
        assert np.abs(want).max() > 0
    if deterministic:
        again = gpu_adjoint(renderer, problem, params, vis, grad, True)
        for name in got:
            assert np.array_equal(got[name].view(np.uint32), again[name].view(np.uint32)), f"{name} changed between runs"


def test_fp64_gradient_equals_finite_differences(ctx):
    """Central differences of the FP64 loss at the GPU's visibility, for sampled parameters of
    every group, against the FP64 analytic gradient and the GPU adjoint."""
    import torch
    from diff_harness import make_renderer
    from oracle import diff64
    problem = small_problem(seed=8)
    _, renderer, cameras, params = make_renderer(ctx, problem)
    images, vis = run_forward(renderer, cameras, problem, params)
    targets = images.cpu().numpy() * 0.9 + 0.02
    shading = diff64.Shading(problem.mesh, vis.cpu().numpy().view(np.uint32), problem.texture.shape)
    g64 = shading.gradients(problem.texture, problem.vertex_colors, problem.light, problem.ambient,
                            diff64.l2_grad(images.cpu().numpy(), targets))
    grad = torch.tensor(diff64.l2_grad(images.cpu().numpy(), targets).astype(np.float32), device="cuda")
    got = gpu_adjoint(renderer, problem, params, vis, grad, False)
    base = {"texture": problem.texture.astype(np.float64), "vertex_colors": problem.vertex_colors.astype(np.float64),
            "light": problem.light.astype(np.float64)}
    rng = np.random.default_rng(0)
    h = 1e-4
    for gi, name in enumerate(("texture", "vertex_colors", "light")):
        flat_g = g64[gi].reshape(-1)
        touched = np.nonzero(flat_g)[0]
        picks = rng.choice(touched, size=min(8, len(touched)), replace=False)
        for idx in picks:
            plus = {k: v.copy() for k, v in base.items()}
            minus = {k: v.copy() for k, v in base.items()}
            plus[name].reshape(-1)[idx] += h
            minus[name].reshape(-1)[idx] -= h
            fd = (shading.loss(plus["texture"], plus["vertex_colors"], plus["light"], problem.ambient, targets) -
                  shading.loss(minus["texture"], minus["vertex_colors"], minus["light"], problem.ambient, targets)) / (2 * h)
            tol = 1e-4 if name == "light" else 1e-6  # the light's max(0, .) has a kink
            assert abs(fd - flat_g[idx]) <= tol * abs(fd) + 1e-12, f"{name}[{idx}]: fd {fd} analytic {flat_g[idx]}"
            gpu = got[name].reshape(-1)[idx]
            assert abs(gpu - fd) <= GRAD_TOLERANCE * abs(fd) + 1e-7, f"{name}[{idx}]: gpu {gpu} fd {fd}"


def test_autograd_function_harness(ctx):
    """A torch loss back-propagated through the autograd wrapper gives the direct adjoint's gradients."""
    import torch
    from diff_harness import make_renderer, render_function
    problem = small_problem(seed=9)
    _, renderer, cameras, params = make_renderer(ctx, problem)
    Render = render_function()
    leaves = {k: v.clone().requires_grad_(True) for k, v in params.items()}
    targets = torch.full((len(cameras), problem.height, problem.width, 4), 0.25, device="cuda")
    images, vis = Render.apply(leaves["texture"], leaves["vertex_colors"], leaves["light"], renderer, cameras,
                               problem.mesh.model_to_world, True)
    loss = ((images - targets) ** 2).mean()
    loss.backward()
    grad = (2.0 * (images.detach() - targets) / images.numel()).contiguous()
    direct = gpu_adjoint(renderer, problem, params, vis, grad, True)
    for name in leaves:
        np.testing.assert_allclose(leaves[name].grad.cpu().numpy(), direct[name], rtol=1e-5, atol=1e-9)


def test_forward_matches_reference_rgbamultiply_with_unit_light(ctx):
    """Light factor 1 (ambient 1, intensity 0), a one-level texture: the float forward pass times
    255 against the reference's U8 colours from the oracle (same coverage; the reference mixes
    texels in 8 bits and truncates when packing, hence the tolerance of 3)."""
    import torch
    import dfpsr_gb300 as d
    from oracle import port
    scene = scenes.random_triangles(seed=31, triangles=600, width=160, height=120, texture_size=64)
    scene.diffuse_levels = 1
    rc, rd, _ = port.render(scene)
    model = d.Model(ctx, scene)
    renderer = d.Diff(ctx, model, 64, 64, 1.0)
    texels = scene.diffuse.view(np.uint8).reshape(64, 64, 4).astype(np.float32) / 255.0
    points = np.asarray(scene.poly_indices)[:, :3].reshape(-1)
    vcol = np.zeros((len(scene.positions), 4), np.float32)
    vcol[points] = np.asarray(scene.colors)[:, :3, :].reshape(-1, 4)
    params = {"texture": torch.tensor(texels, device="cuda"), "vertex_colors": torch.tensor(vcol, device="cuda"),
              "light": torch.tensor([0.0, 0.0, 1.0, 0.0], device="cuda")}
    images = torch.empty((1, 120, 160, 4), device="cuda")
    vis = torch.empty((1, 120, 160, 3), dtype=torch.int32, device="cuda")
    renderer.forward([model.camera], scene.model_to_world, params["texture"], params["vertex_colors"], params["light"], images, vis)
    covered = vis[0, ..., 0].cpu().numpy().view(np.uint32) != 0xFFFFFFFF
    assert np.array_equal(covered, rd > 0)
    ours = images[0].cpu().numpy() * 255.0
    ref = rc.view(np.uint8).reshape(120, 160, 4).astype(np.float64)
    diff = np.abs(ours - ref)[covered]
    assert diff.max() <= 3.0, f"max {diff.max()}"
    assert diff.mean() < 1.0
