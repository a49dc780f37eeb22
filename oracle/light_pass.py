"""The isometric deferred-light pass on the CPU oracle (test infrastructure; the product never calls
it): the same steps as the GPU pass, each one the oracle's restatement of the reference function,
in the reference's order (sprites one after another, every point light one after another)."""
from __future__ import annotations

import dataclasses
from concurrent.futures import ThreadPoolExecutor

import numpy as np

from . import port

BACKGROUND_HEIGHT = -1000.0


def shadow_cubes(scene, view, workers: int = 1):
    """Every light's six faces (model_renderDepth of the caster from the light), on `workers` threads
    (the faces are independent; each is one call into the oracle, which releases the interpreter)."""
    normal_to_world = np.ctypeslib.as_array(view.normalToWorld).copy()
    res = scene.cube_resolution

    def face(job):
        light, side = job
        transform = np.array([-light["position"][0], -light["position"][1], -light["position"][2], 1, 0, 0, 0, 1, 0, 0, 0, 1],
                             np.float32)
        s = dataclasses.replace(scene.caster, camera_location=port.shadow_side(normal_to_world, side),
                                model_to_world=transform, width=res, height=res, perspective=True, slope=1.0,
                                near_clip=0.01, far_clip=1000.0)
        depth, _ = port.render_depth(s)
        return depth

    jobs = [(light, side) for light in scene.lights for side in range(6)]
    if workers > 1:
        with ThreadPoolExecutor(max_workers=workers) as pool:
            faces = list(pool.map(face, jobs))
    else:
        faces = [face(j) for j in jobs]
    return [np.concatenate(faces[6 * k:6 * k + 6], axis=0) for k in range(len(scene.lights))]


def draw_sprites(scene):
    H, W = scene.height, scene.width
    height = np.full((H, W), BACKGROUND_HEIGHT, np.float32)
    diffuse = np.zeros((H, W), np.uint32)
    normal = np.zeros((H, W), np.uint32)
    sources = [(np.ascontiguousarray(h, np.float32), np.ascontiguousarray(c, np.uint32), np.ascontiguousarray(n, np.uint32))
               for h, c, n in zip(scene.sprite_heights, scene.sprite_diffuse, scene.sprite_normals)]
    for t, left, top, offset_bits in scene.placements:
        offset = float(np.array([offset_bits], np.int32).view(np.float32)[0])
        sh, sc, sn = sources[int(t)]
        port.draw_higher_in_place((height, diffuse, 0, normal, 0), (sh, sc, 0, sn, 0), int(left), int(top), offset)
    return height, diffuse, normal


def run(scene, threads: int, workers: int = 1):
    """Returns (output, light, height, diffuse, normal, cubes).  threads: the reference thread count
    whose row bands the point lights follow; workers: host threads for the shadow faces."""
    view = port.ortho_view(scene.camera_tilt, scene.pixels_per_tile, scene.view_index)
    height, diffuse, normal = draw_sprites(scene)
    cubes = shadow_cubes(scene, view, workers)
    light = np.zeros_like(diffuse)
    light = port.directed_light(view, light, normal, scene.sun_direction, scene.sun_intensity, scene.sun_color, False)
    for l, cube in zip(scene.lights, cubes):
        light = port.point_light(view, scene.center, light, normal, height, l["position"], l["radius"], l["intensity"],
                                 l["color"], cube, threads)
    output = port.blend_light(0, diffuse, light)
    return output, light, height, diffuse, normal, cubes
