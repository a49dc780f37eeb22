"""FP64 host oracle of the differentiable renderer (test infrastructure; the product never calls it).

The differentiable form has no counterpart in the reference, so its oracle re-shades in float64
at fixed coverage: given a visibility buffer (per pixel the fan triangle and the vertex weights
wb, wc that the GPU's forward pass found), it evaluates the shading model stated in
include/dsrg.h in float64, the exact gradient of an L2 loss with respect to every parameter,
and central finite differences of that float64 loss.

Two quantities are kept in binary32 on purpose, because they select discrete things rather than
being smooth functions of the parameters: the texture coordinate u, v (computed from the weights
in float32 exactly as the GPU does, so the same texels and 1/256 sub-texel weights are chosen)
and wa = 1 - (wb + wc).  Everything that depends on the parameters is float64.

The fan-triangle order and corner rule follow the reference's Model::render (model/Model.cpp:135-162):
polygon p gives triangle 0-1-2 and, for quads, 0-2-3.
"""
from __future__ import annotations

import numpy as np

NO_TRIANGLE = 0xFFFFFFFF


def fan_triangles(poly_indices: np.ndarray):
    """(triangle count, 3) polygon-corner slots (polygon * 4 + corner) in fan order."""
    slots = []
    for p, idx in enumerate(np.asarray(poly_indices)):
        slots.append((p * 4, p * 4 + 1, p * 4 + 2))
        if idx[3] >= 0:
            slots.append((p * 4, p * 4 + 2, p * 4 + 3))
    return np.asarray(slots, np.int64).reshape(-1, 3)


def world_normals(positions, poly_indices, model_to_world, slots):
    """Unit (B - A) x (C - A) of every fan triangle in world space, float64."""
    m = np.asarray(model_to_world, np.float64)
    axes = np.stack([m[3:6], m[6:9], m[9:12]])  # rows: x, y, z axes
    world = np.asarray(positions, np.float64) @ axes + m[0:3]
    pts = np.asarray(poly_indices).reshape(-1)[slots]
    a, b, c = world[pts[:, 0]], world[pts[:, 1]], world[pts[:, 2]]
    n = np.cross(b - a, c - a)
    length = np.linalg.norm(n, axis=1, keepdims=True)
    return np.where(length > 0, n / np.where(length > 0, length, 1.0), 0.0)


class Shading:
    """Everything of the visible pixels that does not depend on the parameters."""

    def __init__(self, mesh, visibility: np.ndarray, texture_shape):
        vis = np.asarray(visibility).reshape(-1, 3)
        self.pixels = vis.shape[0]
        self.valid = np.nonzero(vis[:, 0] != NO_TRIANGLE)[0]
        tri = vis[self.valid, 0].astype(np.int64)
        wb = vis[self.valid, 1].view(np.float32)
        wc = vis[self.valid, 2].view(np.float32)
        wa = (np.float32(1.0) - (wb + wc)).astype(np.float32)
        self.slots_all = fan_triangles(mesh.poly_indices)
        slots = self.slots_all[tri]
        self.tri = tri
        self.points = np.asarray(mesh.poly_indices).reshape(-1)[slots]          # (n, 3)
        self.weights = np.stack([wa, wb, wc], axis=1).astype(np.float64)        # (n, 3)
        uv = np.asarray(mesh.tex_coords, np.float32).reshape(-1, 4)[:, :2][slots]  # (n, 3, 2) float32
        w32 = np.stack([wa, wb, wc], axis=1)
        u = ((uv[:, 0, 0] * w32[:, 0]) + (uv[:, 1, 0] * w32[:, 1])) + (uv[:, 2, 0] * w32[:, 2])
        v = ((uv[:, 0, 1] * w32[:, 0]) + (uv[:, 1, 1] * w32[:, 1])) + (uv[:, 2, 1] * w32[:, 2])
        th, tw = texture_shape[0], texture_shape[1]
        lw, lh = int(tw).bit_length() - 1, int(th).bit_length() - 1

        def sub(coord, log2):
            scaled = ((coord.astype(np.float32) + np.float32(256.0)) * np.float32(256 << log2)).astype(np.float32)
            return (scaled.astype(np.float64).astype(np.int64) & 0xFFFFFFFF) - 128 & 0xFFFFFFFF

        sx, sy = sub(u, lw), sub(v, lh)
        fx, fy = (sx & 255) / 256.0, (sy & 255) / 256.0
        left, right = (sx >> 8) & (tw - 1), ((sx >> 8) + 1) & (tw - 1)
        top, bottom = (sy >> 8) & (th - 1), ((sy >> 8) + 1) & (th - 1)
        self.taps = np.stack([top * tw + left, top * tw + right, bottom * tw + left, bottom * tw + right], axis=1)
        self.tap_weights = np.stack([(1 - fx) * (1 - fy), fx * (1 - fy), (1 - fx) * fy, fx * fy], axis=1)
        self.normals_all = world_normals(mesh.positions, mesh.poly_indices, mesh.model_to_world, self.slots_all)
        self.normals = self.normals_all[tri]

    def forward(self, texture, vertex_colors, light, ambient):
        tex = np.asarray(texture, np.float64).reshape(-1, 4)
        vcol = np.asarray(vertex_colors, np.float64)
        light = np.asarray(light, np.float64)
        texel = np.einsum("nk,nkc->nc", self.tap_weights, tex[self.taps])
        vertex = np.einsum("ni,nic->nc", self.weights, vcol[self.points])
        ndl = -(self.normals @ light[:3])
        factor = ambient + light[3] * np.maximum(ndl, 0.0)
        out = np.zeros((self.pixels, 4))
        rgb = texel[:, :3] * vertex[:, :3] * factor[:, None]
        out[self.valid, :3] = rgb
        out[self.valid, 3] = texel[:, 3] * vertex[:, 3]
        return out, (texel, vertex, ndl, factor)

    def loss(self, texture, vertex_colors, light, ambient, targets):
        out, _ = self.forward(texture, vertex_colors, light, ambient)
        d = out - np.asarray(targets, np.float64).reshape(-1, 4)
        return float(np.sum(d * d) / d.size)

    def gradients(self, texture, vertex_colors, light, ambient, grad_images):
        """dL/dtexture, dL/dvertex colours and dL/dlight for dL/dimages = grad_images."""
        tex = np.asarray(texture, np.float64)
        vcol = np.asarray(vertex_colors, np.float64)
        light = np.asarray(light, np.float64)
        _, (texel, vertex, ndl, factor) = self.forward(tex, vcol, light, ambient)
        g = np.asarray(grad_images, np.float64).reshape(-1, 4)[self.valid]
        lit = np.concatenate([np.repeat(factor[:, None], 3, axis=1), np.ones((len(factor), 1))], axis=1)
        gt = g * vertex * lit
        gc = g * texel * lit
        gtex = np.zeros((tex.shape[0] * tex.shape[1], 4))
        for k in range(4):
            for ch in range(4):
                gtex[:, ch] += np.bincount(self.taps[:, k], weights=gt[:, ch] * self.tap_weights[:, k], minlength=gtex.shape[0])
        gv = np.zeros_like(vcol)
        for i in range(3):
            for ch in range(4):
                gv[:, ch] += np.bincount(self.points[:, i], weights=gc[:, ch] * self.weights[:, i], minlength=len(vcol))
        dfactor = np.sum(g[:, :3] * texel[:, :3] * vertex[:, :3], axis=1)
        on = ndl > 0
        glight = np.zeros(4)
        glight[:3] = -np.sum((dfactor * light[3] * on)[:, None] * self.normals, axis=0)
        glight[3] = np.sum(dfactor * ndl * on)
        return gtex.reshape(tex.shape), gv, glight


def l2_grad(images, targets):
    d = np.asarray(images, np.float64) - np.asarray(targets, np.float64)
    return 2.0 * d / d.size


def relative_error(got, want) -> float:
    got = np.asarray(got, np.float64).reshape(-1)
    want = np.asarray(want, np.float64).reshape(-1)
    scale = np.linalg.norm(want)
    return float(np.linalg.norm(got - want) / scale) if scale > 0 else float(np.linalg.norm(got))
