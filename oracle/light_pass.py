"""The isometric deferred-light pass on the CPU oracle (test infrastructure; the product never calls
it): the same steps as the GPU pass, each one the oracle's restatement of the reference function,
in the reference's order (sprites one after another, every point light one after another)."""
from __future__ import annotations

import dataclasses

import numpy as np

from . import port

BACKGROUND_HEIGHT = -1000.0


def shadow_cubes(scene, view):
    normal_to_world = np.ctypeslib.as_array(view.normalToWorld).copy()
    res = scene.cube_resolution
    cubes = []
    for light in scene.lights:
        transform = np.array([-light["position"][0], -light["position"][1], -light["position"][2], 1, 0, 0, 0, 1, 0, 0, 0, 1],
                             np.float32)
        faces = []
        for side in range(6):
            s = dataclasses.replace(scene.caster, camera_location=port.shadow_side(normal_to_world, side),
                                    model_to_world=transform, width=res, height=res, perspective=True, slope=1.0,
                                    near_clip=0.01, far_clip=1000.0)
            depth, _ = port.render_depth(s)
            faces.append(depth)
        cubes.append(np.concatenate(faces, axis=0))
    return cubes


def draw_sprites(scene):
    H, W = scene.height, scene.width
    height = np.full((H, W), BACKGROUND_HEIGHT, np.float32)
    diffuse = np.zeros((H, W), np.uint32)
    normal = np.zeros((H, W), np.uint32)
    for t, left, top, offset_bits in scene.placements:
        offset = float(np.array([offset_bits], np.int32).view(np.float32)[0])
        height, diffuse, normal = port.draw_higher(
            (height, diffuse, 0, normal, 0),
            (scene.sprite_heights[t], scene.sprite_diffuse[t], 0, scene.sprite_normals[t], 0), int(left), int(top), offset)
    return height, diffuse, normal


def run(scene, threads: int):
    """Returns (output, light, height, diffuse, normal, cubes)."""
    view = port.ortho_view(scene.camera_tilt, scene.pixels_per_tile, scene.view_index)
    height, diffuse, normal = draw_sprites(scene)
    cubes = shadow_cubes(scene, view)
    light = np.zeros_like(diffuse)
    light = port.directed_light(view, light, normal, scene.sun_direction, scene.sun_intensity, scene.sun_color, False)
    for l, cube in zip(scene.lights, cubes):
        light = port.point_light(view, scene.center, light, normal, height, l["position"], l["radius"], l["intensity"],
                                 l["color"], cube, threads)
    output = port.blend_light(0, diffuse, light)
    return output, light, height, diffuse, normal, cubes
