"""Seeded synthetic scenes for the DFPSR triangle path.

Every scene is plain numpy data laid out like the reference's Model
(Source/DFPSR/implementation/render/model/Model.h:54-64): indexed positions,
polygons of 3 or 4 corners with a texture coordinate (u1, v1, u2, v2) and an
RGBA colour per corner, one part with an optional diffuse and light texture.
The same arrays feed the GPU renderer, the CPU oracle and the reference build,
so the three render identical inputs.
"""
from __future__ import annotations

import dataclasses
import math
from typing import Optional

import numpy as np


@dataclasses.dataclass
class Scene:
    width: int
    height: int
    positions: np.ndarray          # (N, 3) float32, model space
    poly_indices: np.ndarray       # (P, 4) int32, index 3 is -1 for triangles
    tex_coords: np.ndarray         # (P, 4, 4) float32 (u1, v1, u2, v2) per corner
    colors: np.ndarray             # (P, 4, 4) float32 RGBA per corner
    diffuse: Optional[np.ndarray]  # (H, W) uint32 level-0 texels, RGBA bytes in memory order
    diffuse_levels: int
    light: Optional[np.ndarray]
    light_levels: int
    filter: int                    # 0 Solid, 1 Alpha
    camera_location: np.ndarray    # (12,) float32: position, xAxis, yAxis, zAxis
    perspective: bool
    slope: float                   # widthSlope (perspective) or halfWidth (orthogonal)
    near_clip: float
    far_clip: float
    model_to_world: np.ndarray     # (12,) float32

    @property
    def triangle_count(self) -> int:
        return int(np.sum(np.where(self.poly_indices[:, 3] < 0, 1, 2)))


IDENTITY = np.array([0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0, 1], dtype=np.float32)


def _normalize(v):
    v = np.asarray(v, dtype=np.float64)
    n = np.linalg.norm(v)
    return v / n if n > 0 else np.array([0.0, 0.0, 1.0])


def axis_system(forward, up):
    """Camera axes like FMatrix3x3::makeAxisSystem (math/FMatrix3x3.h:46-53), in float64."""
    z = _normalize(forward)
    x = _normalize(np.cross(_normalize(up), z))
    y = _normalize(np.cross(z, x))
    return x, y, z


def camera_location(position, forward, up=(0.0, 1.0, 0.0)) -> np.ndarray:
    x, y, z = axis_system(forward, up)
    return np.concatenate([np.asarray(position, np.float64), x, y, z]).astype(np.float32)


def noise_texture(rng: np.random.Generator, size: int) -> np.ndarray:
    return rng.integers(0, 2**32, size=(size, size), dtype=np.uint64).astype(np.uint32)


def random_triangles(seed: int = 1234, triangles: int = 20000, width: int = 800, height: int = 600,
                     texture_size: int = 256, fov_degrees: float = 60.0) -> Scene:
    """Independent triangles with corners uniform in [-1, 1]^3, seen from distance 3.

    Per-vertex RGBA colours are uniform bytes divided by 255, texture coordinates
    uniform in [0, 1], and one uniform-noise texture with a full mip chain.
    """
    rng = np.random.default_rng(seed)
    positions = rng.uniform(-1.0, 1.0, size=(triangles * 3, 3)).astype(np.float32)
    idx = np.arange(triangles * 3, dtype=np.int32).reshape(triangles, 3)
    poly = np.concatenate([idx, -np.ones((triangles, 1), np.int32)], axis=1)
    colors = np.zeros((triangles, 4, 4), np.float32)
    colors[:, :3, :] = rng.integers(0, 256, size=(triangles, 3, 4)).astype(np.float32) / np.float32(255.0)
    tex = np.zeros((triangles, 4, 4), np.float32)
    tex[:, :3, :] = rng.uniform(0.0, 1.0, size=(triangles, 3, 4)).astype(np.float32)
    diffuse = noise_texture(rng, texture_size) if texture_size else None
    slope = np.float32(math.tan(math.radians(fov_degrees) * 0.5))
    return Scene(width, height, positions, poly, tex, colors, diffuse, 16, None, 1, 0,
                 camera_location((0.0, 0.0, -3.0), (0.0, 0.0, 1.0)), True, float(slope), 0.01, 1000.0,
                 IDENTITY.copy())


BATCH_RESOLUTIONS = ((64, 64), (256, 256), (640, 480), (1024, 768))


def batch_frames(seed: int = 4321, frames: int = 256, resolutions=BATCH_RESOLUTIONS, min_triangles: int = 1000,
                 max_triangles: int = 200000, texture_size: int = 256) -> list:
    """The mixed-size batch: every frame a random_triangles scene with its own seed and its own
    noise texture, a resolution drawn uniformly from `resolutions` and a triangle count drawn
    log-uniformly from [min_triangles, max_triangles]."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(frames):
        w, h = resolutions[int(rng.integers(0, len(resolutions)))]
        n = int(round(math.exp(rng.uniform(math.log(min_triangles), math.log(max_triangles)))))
        out.append(random_triangles(seed=int(rng.integers(0, 2**31 - 1)), triangles=n, width=w, height=h,
                                    texture_size=texture_size))
    return out


def value_noise(rng: np.random.Generator, size: int, octaves: int = 6, base_cells: int = 4) -> np.ndarray:
    """Sum of `octaves` layers of bilinearly smoothed lattice noise in [0, 1), float64."""
    result = np.zeros((size, size), np.float64)
    amplitude, total = 1.0, 0.0
    coords = np.arange(size, dtype=np.float64) / size
    for o in range(octaves):
        cells = base_cells << o
        lattice = rng.uniform(0.0, 1.0, size=(cells + 1, cells + 1))
        f = coords * cells
        i0 = np.floor(f).astype(np.int64)
        t = f - i0
        t = t * t * (3.0 - 2.0 * t)
        a = lattice[np.ix_(i0, i0)]
        b = lattice[np.ix_(i0, i0 + 1)]
        c = lattice[np.ix_(i0 + 1, i0)]
        d = lattice[np.ix_(i0 + 1, i0 + 1)]
        ty, tx = t[:, None], t[None, :]
        layer = (a * (1 - tx) + b * tx) * (1 - ty) + (c * (1 - tx) + d * tx) * ty
        result += amplitude * layer
        total += amplitude
        amplitude *= 0.5
    return result / total


def terrain(seed: int = 1234, grid: int = 512, width: int = 1920, height: int = 1080, texture_size: int = 1024,
            height_scale: float = 48.0, pitch_degrees: float = 30.0, camera_height: float = 120.0,
            width_slope: float = 1.0) -> Scene:
    """A grid x grid height field of quads (A-B-C-D with alternating diagonals, as the
    reference's terrain sample builds it: Source/SDK/terrain/main.cpp:121-171), textured
    with seeded noise and coloured with seeded per-point colours, seen from above at a pitch."""
    rng = np.random.default_rng(seed)
    heights = (value_noise(rng, grid) * height_scale).astype(np.float32)
    zs, xs = np.meshgrid(np.arange(grid, dtype=np.float32), np.arange(grid, dtype=np.float32), indexing="ij")
    positions = np.stack([xs, heights, -zs], axis=-1).reshape(-1, 3).astype(np.float32)
    point_colors = np.concatenate([rng.uniform(0.55, 1.0, size=(grid * grid, 3)), np.ones((grid * grid, 1))], axis=1).astype(np.float32)
    px, pz = np.meshgrid(np.arange(1, grid), np.arange(1, grid), indexing="xy")
    px = px.reshape(-1).astype(np.int64); pz = pz.reshape(-1).astype(np.int64)
    x0, z0 = px - 1, pz - 1
    ia = x0 + z0 * grid
    ib = px + z0 * grid
    ic = px + pz * grid
    idd = x0 + pz * grid
    scale = np.float32(1.0) / np.float32(grid - 1.0)
    ta = np.stack([x0 * scale, z0 * scale], -1)
    tb = np.stack([px * scale, z0 * scale], -1)
    tc = np.stack([px * scale, pz * scale], -1)
    td = np.stack([x0 * scale, pz * scale], -1)
    even = ((px + pz) % 2) == 0
    idx = np.where(even[:, None], np.stack([ia, ib, ic, idd], -1), np.stack([ib, ic, idd, ia], -1)).astype(np.int32)
    uv = np.where(even[:, None, None], np.stack([ta, tb, tc, td], 1), np.stack([tb, tc, td, ta], 1)).astype(np.float32)
    tex = np.zeros((idx.shape[0], 4, 4), np.float32)
    tex[:, :, :2] = uv
    colors = point_colors[idx]
    diffuse = noise_texture(rng, texture_size)
    pitch = math.radians(pitch_degrees)
    center = grid * 0.5
    position = (center, camera_height, camera_height / math.tan(pitch) * 0.5)
    forward = (0.0, -math.sin(pitch), -math.cos(pitch))
    return Scene(width, height, positions, idx, tex, colors, diffuse, 16, None, 1, 0,
                 camera_location(position, forward), True, float(width_slope), 0.01, 1000.0, IDENTITY.copy())


def with_variant(scene: Scene, *, texture: bool = True, light: bool = False, colors: str = "random",
                 seed: int = 7, pyramid: bool = True) -> Scene:
    """Same geometry with another RgbaMultiply variant (Source/DFPSR/implementation/render/shader/RgbaMultiply.h:110-173).

    colors: "random" (vertex fading), "white" (colorless), "constant" (one colour per triangle).
    """
    rng = np.random.default_rng(seed)
    s = dataclasses.replace(scene)
    p = scene.colors.shape[0]
    if colors == "white":
        s.colors = np.ones_like(scene.colors)
    elif colors == "constant":
        c = rng.integers(0, 256, size=(p, 1, 4)).astype(np.float32) / np.float32(255.0)
        s.colors = np.repeat(c, 4, axis=1).astype(np.float32)
    if not texture:
        s.diffuse = None
    elif s.diffuse is None:
        s.diffuse = noise_texture(rng, 64)
    if not pyramid:
        s.diffuse_levels = 1
    if light:
        s.light = noise_texture(rng, 32)
        s.light_levels = 1
        t = s.tex_coords.copy()
        t[:, :, 2:] = rng.uniform(0.0, 1.0, size=t[:, :, 2:].shape).astype(np.float32)
        s.tex_coords = t
    else:
        s.light = None
    return s


def torus(major_segments: int = 250, minor_segments: int = 100, major_radius: float = 1.0, minor_radius: float = 0.4,
          uv_repeat: float = 4.0, width: int = 256, height: int = 256, inside_out: bool = False) -> Scene:
    """A closed torus of major x minor quads (2 fan triangles each, 50,000 triangles at 250 x 100)
    around the y axis, with texture coordinates running uv_repeat times around the ring and once
    around the tube (per polygon corner, so the seams need no duplicated points).  The corners
    wind so that the outer surface is front-facing (inside_out turns it around)."""
    i = np.arange(major_segments)
    j = np.arange(minor_segments)
    theta = 2.0 * np.pi * i / major_segments
    phi = 2.0 * np.pi * j / minor_segments
    ring = major_radius + minor_radius * np.cos(phi)[None, :]
    x = ring * np.cos(theta)[:, None]
    z = ring * np.sin(theta)[:, None]
    y = np.broadcast_to(minor_radius * np.sin(phi)[None, :], x.shape)
    positions = np.stack([x, y, z], axis=-1).reshape(-1, 3).astype(np.float32)
    ii, jj = np.meshgrid(i, j, indexing="ij")
    ii, jj = ii.reshape(-1), jj.reshape(-1)
    i1, j1 = (ii + 1) % major_segments, (jj + 1) % minor_segments
    a, b, c, d = ii * minor_segments + jj, i1 * minor_segments + jj, i1 * minor_segments + j1, ii * minor_segments + j1
    flip = not inside_out
    corners = np.stack([a, d, c, b] if flip else [a, b, c, d], axis=1).astype(np.int32)
    cu = np.stack([ii, ii + 1, ii + 1, ii], axis=1).astype(np.float64) * (uv_repeat / major_segments)
    cv = np.stack([jj, jj, jj + 1, jj + 1], axis=1).astype(np.float64) / minor_segments
    if flip:
        cu, cv = cu[:, [0, 3, 2, 1]], cv[:, [0, 3, 2, 1]]
    tex = np.zeros((len(corners), 4, 4), np.float32)
    tex[:, :, 0] = cu
    tex[:, :, 1] = cv
    tex[:, :, 2] = cu
    tex[:, :, 3] = cv
    colors = np.ones((len(corners), 4, 4), np.float32)
    slope = np.float32(math.tan(math.radians(60.0) * 0.5))
    return Scene(width, height, positions, corners, tex, colors, None, 1, None, 1, 0,
                 camera_location((0.0, 0.0, -3.5), (0.0, 0.0, 1.0)), True, float(slope), 0.01, 1000.0, IDENTITY.copy())


def orbit_cameras(seed: int, views: int, distance: float = 3.2) -> list:
    """Camera locations on a sphere around the origin, looking at it, from seeded directions."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(views):
        d = rng.normal(size=3)
        d /= np.linalg.norm(d)
        if abs(d[1]) > 0.95:
            d[1] = 0.95 * np.sign(d[1])
            d /= np.linalg.norm(d)
        out.append(camera_location(tuple(d * distance), tuple(-d)))
    return out


@dataclasses.dataclass
class DiffProblem:
    """The differentiable-rendering workload: a mesh, views, parameters and the perturbed
    parameters that render the target images."""
    mesh: Scene
    cameras: list                 # camera locations (12 floats each)
    width: int
    height: int
    texture: np.ndarray           # (T, T, 4) float32
    vertex_colors: np.ndarray     # (points, 4) float32
    light: np.ndarray             # (4,) float32: dir xyz, intensity
    ambient: float
    target_texture: np.ndarray
    target_vertex_colors: np.ndarray
    target_light: np.ndarray


def diff_problem(seed: int = 99, views: int = 64, size: int = 256, texture_size: int = 512, major: int = 250,
                 minor: int = 100, sigma: float = 0.05) -> DiffProblem:
    rng = np.random.default_rng(seed)
    mesh = torus(major, minor, width=size, height=size)
    cams = orbit_cameras(seed + 1, views)
    tex = (value_noise(rng, texture_size, octaves=5, base_cells=8)[..., None] * 0.6 + 0.2
           + rng.uniform(-0.1, 0.1, size=(texture_size, texture_size, 4))).astype(np.float32)
    tex[..., 3] = 1.0
    vcol = rng.uniform(0.5, 1.0, size=(len(mesh.positions), 4)).astype(np.float32)
    vcol[:, 3] = 1.0
    direction = rng.normal(size=3)
    direction /= np.linalg.norm(direction)
    light = np.array([*direction, 0.8], np.float32)
    t_tex = (tex + rng.normal(0.0, sigma, size=tex.shape)).astype(np.float32)
    t_vcol = (vcol + rng.normal(0.0, sigma, size=vcol.shape)).astype(np.float32)
    t_light = (light + rng.normal(0.0, sigma, size=4)).astype(np.float32)
    return DiffProblem(mesh, cams, size, size, tex, vcol, light, 0.3, t_tex, t_vcol, t_light)


@dataclasses.dataclass
class LightScene:
    """The isometric deferred-light workload: sprite images drawn with draw_higher, point lights with
    shadow cube maps rendered from a caster model, a directed light and blendLight."""
    width: int
    height: int
    camera_tilt: float
    pixels_per_tile: int
    view_index: int
    center: tuple                  # worldCenter in pixels
    sprite_heights: list           # (s, s) float32 per sprite type
    sprite_diffuse: list           # (s, s) uint32 RGBA per sprite type
    sprite_normals: list           # (s, s) uint32 RGBA per sprite type
    placements: np.ndarray         # (n, 4): type, left, top, and the height offset's bits (float32 viewed as int32)
    lights: list                   # dicts: position, radius, intensity, color
    sun_direction: tuple
    sun_intensity: float
    sun_color: tuple
    caster: Scene                  # shadow caster model (positions in tiles, relative to the camera)
    cube_resolution: int


def _sprite_type(rng, size):
    yy, xx = np.mgrid[0:size, 0:size].astype(np.float64)
    c = (size - 1) / 2.0
    r = np.sqrt((xx - c) ** 2 + (yy - c) ** 2) / (size / 2.0)
    dome = np.clip(1.0 - r * r, 0.0, None)
    height = (dome * rng.uniform(1.0, 3.0) + rng.uniform(0.0, 0.15, size=(size, size)) * (dome > 0)).astype(np.float32)
    height[r > 1.0] = -np.inf  # transparent corners
    gy, gx = np.gradient(np.where(r <= 1.0, height.astype(np.float64), 0.0))
    n = np.stack([-gx, -gy, np.ones_like(gx)], axis=-1)
    n /= np.linalg.norm(n, axis=-1, keepdims=True)
    nb = np.clip(n * 127.0 + 128.0, 0, 255).astype(np.uint32)
    normal = nb[..., 0] | (nb[..., 1] << 8) | (nb[..., 2] << 16) | (np.uint32(255) << 24)
    diffuse = rng.integers(0, 2**32, size=(size, size), dtype=np.uint64).astype(np.uint32) | np.uint32(0xFF000000)
    return height, diffuse, normal.astype(np.uint32)


def light_scene(seed: int = 2024, width: int = 1920, height: int = 1080, sprites: int = 4096, sprite_size: int = 64,
                sprite_types: int = 32, lights: int = 16, radius_px=(100, 400), caster_triangles: int = 2000,
                cube_resolution: int = 512, camera_tilt: float = -0.7, pixels_per_tile: int = 64, view_index: int = 0,
                light_space=None) -> LightScene:
    """Sprites on a grid covering the image (seeded noise images with domed heights), point lights at
    seeded pixel positions with radii uniform in radius_px, and a caster model of small random
    triangles around the lights.  light_space = (screenDepthToLightSpace, normalToWorld) as 3x3 axes
    (row per axis) places the lights; the library's ortho_view provides them."""
    rng = np.random.default_rng(seed)
    types = [_sprite_type(rng, sprite_size) for _ in range(sprite_types)]
    cols = int(math.ceil(math.sqrt(sprites * width / height)))
    rows = int(math.ceil(sprites / cols))
    place = np.zeros((sprites, 4), np.int32)
    for k in range(sprites):
        i, j = k % cols, k // cols
        left = int(round(i * (width + sprite_size) / cols)) - sprite_size // 2 + int(rng.integers(-4, 5))
        top = int(round(j * (height + sprite_size) / rows)) - sprite_size // 2 + int(rng.integers(-4, 5))
        offset = np.float32(j * 0.02 + rng.uniform(0.0, 0.5))
        place[k] = (int(rng.integers(0, sprite_types)), left, top, np.array([offset], np.float32).view(np.int32)[0])
    center = (width // 2, height // 2)
    light_list = []
    if light_space is not None:
        to_light, normal_to_world = (np.asarray(m, np.float64).reshape(3, 3) for m in light_space)
        for _ in range(lights):
            px, py = rng.uniform(0, width), rng.uniform(0, height)
            h = rng.uniform(1.0, 3.0)
            screen = np.array([px - center[0], py - center[1], h])
            ls = screen[0] * to_light[0] + screen[1] * to_light[1] + screen[2] * to_light[2]
            pos = ls[0] * normal_to_world[0] + ls[1] * normal_to_world[1] + ls[2] * normal_to_world[2]
            scale = np.linalg.norm(to_light[0])  # tiles per pixel along the screen's x axis
            radius = float(rng.uniform(*radius_px) * scale)
            color = tuple(int(c) for c in rng.integers(128, 256, size=3))
            light_list.append({"position": tuple(float(v) for v in pos), "radius": radius,
                               "intensity": float(rng.uniform(0.6, 1.2)), "color": color})
    # casters: small triangles scattered around the lights (tile units, relative to the camera)
    anchors = np.array([l["position"] for l in light_list]) if light_list else np.zeros((1, 3))
    a = anchors[rng.integers(0, len(anchors), size=caster_triangles)]
    centers = a + rng.normal(0.0, 1.5, size=(caster_triangles, 3))
    corners = centers[:, None, :] + rng.normal(0.0, 0.35, size=(caster_triangles, 3, 3))
    positions = corners.reshape(-1, 3).astype(np.float32)
    idx = np.arange(caster_triangles * 3, dtype=np.int32).reshape(-1, 3)
    poly = np.concatenate([idx, -np.ones((caster_triangles, 1), np.int32)], axis=1)
    zeros = np.zeros((caster_triangles, 4, 4), np.float32)
    caster = Scene(cube_resolution, cube_resolution, positions, poly, zeros, np.ones_like(zeros), None, 1, None, 1, 0,
                   camera_location((0.0, 0.0, 0.0), (0.0, 0.0, 1.0)), True, 1.0, 0.01, 1000.0, IDENTITY.copy())
    # the sun shines down and away from the camera in light space, so that flat sprite pixels are lit
    sun_light_space = np.array([rng.uniform(-0.4, 0.4), -0.6, -0.75])
    if light_space is not None:
        n = np.asarray(light_space[1], np.float64).reshape(3, 3)
        sun = sun_light_space[0] * n[0] + sun_light_space[1] * n[1] + sun_light_space[2] * n[2]
    else:
        sun = sun_light_space
    return LightScene(width, height, camera_tilt, pixels_per_tile, view_index, center,
                      [t[0] for t in types], [t[1] for t in types], [t[2] for t in types], place, light_list,
                      tuple(float(v) for v in sun / np.linalg.norm(sun)), 0.35, (200, 210, 255), caster, cube_resolution)


BOX_FACES = np.array([[0, 2, 3, 1], [4, 5, 7, 6], [0, 1, 5, 4], [2, 6, 7, 3], [0, 4, 6, 2], [1, 3, 7, 5]], np.int32)


def box_model(rng: np.random.Generator, minimum, maximum, camera: Scene, texture_size: int = 32) -> Scene:
    """A box of six quads facing outwards, random corner colours and texture coordinates, drawn
    with `camera`'s camera and target size."""
    x0, y0, z0 = minimum
    x1, y1, z1 = maximum
    positions = np.array([[x0, y0, z0], [x1, y0, z0], [x0, y1, z0], [x1, y1, z0],
                          [x0, y0, z1], [x1, y0, z1], [x0, y1, z1], [x1, y1, z1]], np.float32)
    colors = rng.integers(64, 256, size=(6, 4, 4)).astype(np.float32) / np.float32(255.0)
    colors[:, :, 3] = 1.0
    tex = rng.uniform(0.0, 1.0, size=(6, 4, 4)).astype(np.float32)
    return dataclasses.replace(camera, positions=positions, poly_indices=BOX_FACES.copy(), tex_coords=tex, colors=colors,
                               diffuse=noise_texture(rng, texture_size), diffuse_levels=16, light=None, filter=0,
                               model_to_world=IDENTITY.copy())


def placed(scene: Scene, translation, rotation=None) -> Scene:
    """The scene with a model-to-world transform (position, then the rotation's x, y and z axes)."""
    r = np.eye(3, dtype=np.float32) if rotation is None else np.asarray(rotation, np.float32)
    t = np.concatenate([np.asarray(translation, np.float32), r[0], r[1], r[2]]).astype(np.float32)
    return dataclasses.replace(scene, model_to_world=t)


def random_rotation(rng: np.random.Generator) -> np.ndarray:
    q, r = np.linalg.qr(rng.normal(size=(3, 3)))
    q = q * np.sign(np.diag(r))
    if np.linalg.det(q) < 0:
        q[:, 0] = -q[:, 0]
    return q.astype(np.float32)


@dataclasses.dataclass
class OcclusionScene:
    """A renderer frame for the occlusion grid: a wall in front of the camera, a field of small
    triangles partly behind it, boxes all over, and a depth image from an earlier pass whose top
    rows can occlude (renderer_occludeFromTopRows)."""
    camera: Scene           # camera and target size (no geometry)
    wall: Scene
    panel: Scene            # a tilted quad that only occludes through its triangles
    field: Scene
    props: list
    depth: np.ndarray       # (height, width) float32 initial depth buffer
    color: np.ndarray       # (height, width) uint32 initial colour buffer

    @staticmethod
    def bound(scene: Scene):
        """The model's bound as the reference keeps it: grown from the origin (Model.cpp:281-288)."""
        p = scene.positions
        return np.minimum(p.min(axis=0), 0.0).astype(np.float32), np.maximum(p.max(axis=0), 0.0).astype(np.float32)


def occlusion_scene(seed: int = 77, width: int = 320, height: int = 240, props: int = 24, field_triangles: int = 1500,
                    perspective: bool = True) -> OcclusionScene:
    rng = np.random.default_rng(seed)
    if perspective:
        slope = float(np.float32(math.tan(math.radians(30.0))))
        cam = Scene(width, height, np.zeros((0, 3), np.float32), np.zeros((0, 4), np.int32), np.zeros((0, 4, 4), np.float32),
                    np.zeros((0, 4, 4), np.float32), None, 16, None, 1, 0, camera_location((0.0, 0.0, -6.0), (0.0, 0.0, 1.0)),
                    True, slope, 0.01, 1000.0, IDENTITY.copy())
    else:
        cam = Scene(width, height, np.zeros((0, 3), np.float32), np.zeros((0, 4), np.int32), np.zeros((0, 4, 4), np.float32),
                    np.zeros((0, 4, 4), np.float32), None, 16, None, 1, 0, camera_location((0.0, 0.0, -6.0), (0.0, 0.0, 1.0)),
                    False, 4.0, 0.01, 1000.0, IDENTITY.copy())
    wall = placed(box_model(rng, (-1.5, -1.0, -0.2), (1.5, 1.0, 0.2), cam), (0.0, -0.2, 0.0))
    panel_points = np.array([[-4.5, 0.6, 2.0], [-1.8, 0.6, 3.5], [-4.5, 3.2, 2.5], [-1.8, 3.2, 4.0]], np.float32)
    panel = dataclasses.replace(cam, positions=panel_points, poly_indices=np.array([[0, 2, 3, 1]], np.int32),
                                tex_coords=rng.uniform(0.0, 1.0, size=(1, 4, 4)).astype(np.float32),
                                colors=np.ones((1, 4, 4), np.float32), diffuse=noise_texture(rng, 32), diffuse_levels=16,
                                filter=0, model_to_world=IDENTITY.copy())
    # the field: small triangles scattered over a slab behind and beside the wall
    n = field_triangles
    centers = np.stack([rng.uniform(-5.0, 5.0, n), rng.uniform(-3.5, 3.5, n), rng.uniform(1.0, 8.0, n)], axis=1)
    corners = centers[:, None, :] + rng.uniform(-0.35, 0.35, size=(n, 3, 3))
    positions = corners.reshape(-1, 3).astype(np.float32)
    idx = np.arange(n * 3, dtype=np.int32).reshape(n, 3)
    poly = np.concatenate([idx, -np.ones((n, 1), np.int32)], axis=1)
    colors = np.zeros((n, 4, 4), np.float32)
    colors[:, :3, :] = rng.integers(0, 256, size=(n, 3, 4)).astype(np.float32) / np.float32(255.0)
    tex = np.zeros((n, 4, 4), np.float32)
    tex[:, :3, :] = rng.uniform(0.0, 1.0, size=(n, 3, 4)).astype(np.float32)
    field = dataclasses.replace(cam, positions=positions, poly_indices=poly, tex_coords=tex, colors=colors,
                                diffuse=noise_texture(rng, 32), diffuse_levels=16, filter=0, model_to_world=IDENTITY.copy())
    prop_list = []
    for _ in range(props):
        h = rng.uniform(0.15, 0.4, 3)
        box = box_model(rng, tuple(-h), tuple(h), cam)
        where = (rng.uniform(-4.0, 4.0), rng.uniform(-2.5, 2.5), rng.uniform(-2.5, 9.0))
        prop_list.append(placed(box, where, random_rotation(rng)))
    # depth of an earlier pass: a near band over the upper left, and near stripes on the top pixel row
    # of every cell of the right half (only those rows occlude from the top rows, so what lies behind
    # the stripes is culled although it shows between them); nothing (0, or the far clear value) elsewhere
    ys, xs = np.mgrid[0:height, 0:width]
    near = ((ys < height * 0.45) & (xs < width * 0.55)) | ((ys % 16 == 0) & (xs >= width * 0.55))
    distance = (3.0 + 4.0 * xs / width).astype(np.float32)
    if perspective:
        depth = np.where(near, np.float32(1.0) / distance, np.float32(0.0)).astype(np.float32)
    else:
        depth = np.where(near, distance, np.float32(1000.0)).astype(np.float32)
    color = rng.integers(0, 2**32, size=(height, width), dtype=np.uint64).astype(np.uint32)
    return OcclusionScene(cam, wall, panel, field, prop_list, depth, color)


@dataclasses.dataclass
class DenseScene:
    """A model drawn by the sprite engine's renderDenseModel into height, diffuse and normal images."""
    positions: np.ndarray        # (N, 3) float32, model space in tiles
    polygons: np.ndarray         # (P, 4) int32, index 3 is -1 for triangles
    colors: np.ndarray           # (P, 4, 4) float32 RGBA per corner, in [0, 1]
    camera_tilt: float
    pixels_per_tile: int
    view_index: int
    origin: tuple                # the world origin in target pixels
    model_to_world: np.ndarray   # (12,) float32
    height: np.ndarray           # (H, W) float32 initial height image
    diffuse: np.ndarray          # (H, W) uint32
    normal: np.ndarray           # (H, W) uint32


def dense_scene(seed: int = 17, width: int = 256, height: int = 192, major: int = 40, minor: int = 16, view_index: int = 0,
                prefilled: bool = False, pixels_per_tile: int = 48) -> DenseScene:
    """A vertex-coloured torus (quads) of one tile's radius, rotated and placed at the centre of the
    image, seen through an ortho view; optionally over a prefilled height and colour image."""
    rng = np.random.default_rng(seed)
    t = torus(major_segments=major, minor_segments=minor, major_radius=1.0, minor_radius=0.35)
    colors = rng.uniform(0.0, 1.0, size=t.colors.shape).astype(np.float32)
    rot = random_rotation(rng)
    model = np.concatenate([rng.uniform(-0.3, 0.3, 3), rot.reshape(-1)]).astype(np.float32)
    h0 = (rng.uniform(-2.0, 1.0, size=(height, width)) if prefilled else np.full((height, width), -1e30)).astype(np.float32)
    d0 = rng.integers(0, 2**32, size=(height, width), dtype=np.uint64).astype(np.uint32) if prefilled else np.zeros((height, width), np.uint32)
    n0 = rng.integers(0, 2**32, size=(height, width), dtype=np.uint64).astype(np.uint32) if prefilled else np.zeros((height, width), np.uint32)
    return DenseScene(t.positions, t.poly_indices, colors, -1.0, pixels_per_tile, view_index, (width * 0.5, height * 0.5), model,
                      h0, d0, n0)
