"""Gradient-check harness of the differentiable renderer: dsrg_diff_forward / dsrg_diff_adjoint
wrapped in a torch.autograd.Function, so that a loss written in torch back-propagates through the
hand-written adjoint.  Test infrastructure only; the library itself has no torch dependency."""
import numpy as np


def make_renderer(ctx, problem):
    import torch
    import dfpsr_gb300 as d
    model = d.Model(ctx, problem.mesh)
    tex_h, tex_w = problem.texture.shape[:2]
    renderer = d.Diff(ctx, model, tex_w, tex_h, problem.ambient)
    cameras = []
    for loc in problem.cameras:
        cam = d.camera_struct(problem.mesh)
        for i in range(12):
            cam.location[i] = float(loc[i])
        cam.width, cam.height = problem.width, problem.height
        cameras.append(cam)
    params = {name: torch.tensor(np.ascontiguousarray(getattr(problem, name)), device="cuda")
              for name in ("texture", "vertex_colors", "light")}
    return model, renderer, cameras, params


def render_function():
    import torch

    class Render(torch.autograd.Function):
        @staticmethod
        def forward(fctx, texture, vertex_colors, light, renderer, cameras, transform, deterministic):
            views, h, w = len(cameras), cameras[0].height, cameras[0].width
            images = torch.empty((views, h, w, 4), dtype=torch.float32, device="cuda")
            visibility = torch.empty((views, h, w, 3), dtype=torch.int32, device="cuda")
            renderer.forward(cameras, transform, texture, vertex_colors, light, images, visibility)
            fctx.save_for_backward(texture, vertex_colors, light, visibility)
            fctx.renderer, fctx.transform, fctx.deterministic = renderer, transform, deterministic
            fctx.shape = (views, h, w)
            fctx.mark_non_differentiable(visibility)
            return images, visibility

        @staticmethod
        def backward(fctx, grad_images, grad_visibility):
            texture, vertex_colors, light, visibility = fctx.saved_tensors
            views, h, w = fctx.shape
            g_tex, g_vcol, g_light = torch.empty_like(texture), torch.empty_like(vertex_colors), torch.empty_like(light)
            fctx.renderer.adjoint(views, w, h, fctx.transform, texture, vertex_colors, light, visibility,
                                  grad_images.contiguous(), g_tex, g_vcol, g_light, fctx.deterministic)
            return g_tex, g_vcol, g_light, None, None, None, None

    return Render
