"""The isometric deferred-light pass on the GPU, through the C ABI: sprites drawn with draw_higher into
height, diffuse and normal images, one shadow cube map per point light rendered with depth-only
batches (six faces per light, all lights in one batch), a directed light, every point light in one
pass, and blendLight into the output image (the steps of the reference's sprite engine frame:
SDK/SpriteEngine/spriteAPI.cpp, lightAPI.cpp)."""
from __future__ import annotations

import numpy as np

from . import Model, SpriteArray, camera_struct, ortho_view, shadow_side_location

BACKGROUND_HEIGHT = -1000.0


class DeferredLightPass:
    """Device resources of one LightScene (uploaded once) and the pass itself (`run`)."""

    def __init__(self, ctx, scene, reference_threads: int = 0):
        import torch
        self.ctx, self.scene, self.threads = ctx, scene, reference_threads
        dev = lambda a, dt: torch.tensor(np.ascontiguousarray(a).view(dt), device="cuda")
        self.view = ortho_view(scene.camera_tilt, scene.pixels_per_tile, scene.view_index)
        self.types = [(dev(h, np.float32), dev(c, np.int32), dev(n, np.int32))
                      for h, c, n in zip(scene.sprite_heights, scene.sprite_diffuse, scene.sprite_normals)]
        sprites = []
        for t, left, top, offset_bits in scene.placements:
            h, c, n = self.types[int(t)]
            sprites.append({"height": h, "color_a": c, "color_b": n, "left": int(left), "top": int(top),
                            "offset": float(np.array([offset_bits], np.int32).view(np.float32)[0])})
        self.sprites = SpriteArray(sprites)  # built once: the call only passes the array
        H, W = scene.height, scene.width
        self.height = torch.empty((H, W), dtype=torch.float32, device="cuda")
        self.diffuse = torch.empty((H, W), dtype=torch.int32, device="cuda")
        self.normal = torch.empty((H, W), dtype=torch.int32, device="cuda")
        self.light = torch.empty((H, W), dtype=torch.int32, device="cuda")
        self.output = torch.empty((H, W), dtype=torch.int32, device="cuda")
        res = scene.cube_resolution
        self.cubes = [torch.empty((6 * res, res), dtype=torch.float32, device="cuda") for _ in scene.lights]
        self.caster = Model(ctx, scene.caster)
        self.shadows = ctx.batch()
        self.shadows.set_depth_only(True)
        normal_to_world = np.ctypeslib.as_array(self.view.normalToWorld).copy()
        for k, light in enumerate(scene.lights):
            transform = np.array([-light["position"][0], -light["position"][1], -light["position"][2],
                                  1, 0, 0, 0, 1, 0, 0, 0, 1], np.float32)
            for side in range(6):
                cam = camera_struct(scene.caster)
                loc = shadow_side_location(normal_to_world, side)
                for i in range(12):
                    cam.location[i] = float(loc[i])
                cam.perspective, cam.slope, cam.nearClip, cam.farClip = 1, 1.0, 0.01, 1000.0
                cam.width = cam.height = res
                frame = self.shadows.add_frame(None, self.cubes[k][side * res:(side + 1) * res])
                self.shadows.give_task(frame, self.caster, cam, transform)
        self.light_list = [dict(l, cube=self.cubes[k]) for k, l in enumerate(scene.lights)]

    def tune_shadows(self, rounds: int = 2) -> dict:
        """Gives the shadow batch a tile-kernel configuration of its own, the autotuner's choice for
        it (cube faces of large triangles suit other shapes than the frames drawn with the
        context's configuration, which stays as it is)."""
        self.shadows.set_tuning(self.ctx.tuning())
        return self.shadows.autotune(rounds)

    def run(self):
        """One frame in one call (dsrg_sprite_frame); returns the output image (device)."""
        s = self.scene
        self.ctx.sprite_frame(self.view, s.center, (self.height, self.diffuse, self.normal, self.light, self.output),
                              (BACKGROUND_HEIGHT, 0, 0), self.sprites, (s.sun_direction, s.sun_intensity, s.sun_color),
                              self.shadows, self.light_list, self.threads)
        return self.output

    def run_steps(self):
        """The same frame as one call per step; returns the output image (device)."""
        s = self.scene
        self.height.fill_(BACKGROUND_HEIGHT)
        self.diffuse.zero_()
        self.normal.zero_()
        for cube in self.cubes:
            cube.zero_()  # CubeMapF32::clear (spriteAPI.cpp:357-359)
        self.ctx.draw_higher(self.height, self.diffuse, self.normal, self.sprites)
        self.shadows.render()
        self.ctx.light_directed(self.view, self.light, self.normal, s.sun_direction, s.sun_intensity, s.sun_color, add=False)
        self.ctx.light_points(self.view, s.center, self.light, self.normal, self.height, self.light_list, self.threads)
        self.ctx.light_blend(self.output, self.diffuse, self.light)
        return self.output

    def destroy(self):
        self.shadows.destroy()
        self.caster.destroy()
