"""ctypes front end of the reference itself, built out-of-tree into oracle/_ref/ -- test infrastructure only.

`available()` is False wherever the reference sources were not present to
build from (for example on a machine that only received this repository).
"""
from __future__ import annotations

import atexit
import ctypes as C
import os
import subprocess
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
# the reference checkout: $DFPSR_REFERENCE, else a directory named `reference` beside the repository
REFERENCE_ROOT = os.environ.get("DFPSR_REFERENCE", os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference"))


def lib_path(variant: str = "exact") -> str:
    return os.path.join(REF_DIR, f"libdsr_ref_{variant}.so")


def build(jobs: int = 8) -> bool:
    """Builds both reference variants when the reference sources exist; returns availability."""
    if not os.path.isdir(os.path.join(REFERENCE_ROOT, "Source", "DFPSR")):
        return available()
    repo = os.path.dirname(HERE)
    subprocess.check_call(["make", "-s", "-f", os.path.join("oracle", "Makefile.ref"), f"REF={REFERENCE_ROOT}", f"-j{jobs}"],
                          cwd=repo)
    return available()


def available(variant: str = "exact") -> bool:
    if not os.path.exists(lib_path(variant)):
        return False
    try:
        _load(variant)
        return True
    except OSError:
        return False


_libs = {}
_shut_down = []


def _shutdown(l):
    _shut_down.append(True)
    l.refh_shutdown()


def _load(variant: str):
    if variant not in _libs:
        l = C.CDLL(lib_path(variant))
        P = C.c_void_p
        l.refh_texture_create.argtypes = [P, C.c_int, C.c_int, C.c_int]
        l.refh_texture_create.restype = P
        l.refh_texture_create_ordered.argtypes = [P, C.c_int, C.c_int, C.c_int, C.c_int]
        l.refh_texture_create_ordered.restype = P
        l.refh_texture_info.argtypes = [P, P, P, C.c_int]
        l.refh_texture_info.restype = C.c_int
        l.refh_texture_free.argtypes = [P]
        l.refh_model_create.argtypes = [P, C.c_int, P, P, P, C.c_int, P, P, C.c_int]
        l.refh_model_create.restype = P
        l.refh_model_free.argtypes = [P]
        l.refh_model_render.argtypes = [P, P, P, C.c_int, C.c_float, C.c_float, C.c_float, C.c_int, C.c_int, P, P,
                                        C.c_int, C.c_int]
        l.refh_model_render.restype = C.c_int
        l.refh_model_render_depth.argtypes = [P, P, P, C.c_int, C.c_float, C.c_float, C.c_float, C.c_int, C.c_int, P]
        l.refh_model_render_depth.restype = C.c_int
        l.refh_camera_to_screen.argtypes = [P, C.c_int, C.c_float, C.c_float, C.c_float, C.c_int, C.c_int, P, P, P]
        l.refh_triangle_rows.argtypes = [P, P, C.c_int, C.c_int, P, P, P, C.c_int]
        l.refh_triangle_rows.restype = C.c_int
        cam = [P, C.c_int, C.c_float, C.c_float, C.c_float, C.c_int, C.c_int]
        l.refh_renderer_create.restype = P
        l.refh_renderer_free.argtypes = [P]
        l.refh_renderer_begin.argtypes = [P, P, P, C.c_int, C.c_int, C.c_int]
        l.refh_renderer_give_task.argtypes = [P, P, P] + cam
        l.refh_renderer_occlude_from_box.argtypes = [P, P, P, P] + cam + [C.c_int]
        l.refh_draw_line.argtypes = [P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_uint32]
        l.refh_renderer_occlude_from_existing_triangles.argtypes = [P]
        l.refh_renderer_give_triangle.argtypes = [P, P, P, P, P, P, P, P, C.c_int] + cam
        l.refh_renderer_occlude_from_top_rows.argtypes = [P] + cam
        l.refh_renderer_is_box_visible.argtypes = [P, P, P, P] + cam
        l.refh_renderer_is_box_visible.restype = C.c_int
        l.refh_renderer_has_occluders.argtypes = [P]
        l.refh_renderer_has_occluders.restype = C.c_int
        l.refh_renderer_end.argtypes = [P, C.c_int]
        atexit.register(_shutdown, l)
        _libs[variant] = l
    return _libs[variant]


def _ptr(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class RefTexture:
    def __init__(self, lib, pixels: np.ndarray, resolutions: int, pack_order: int = 0):
        self.lib = lib
        self.pixels = np.ascontiguousarray(pixels, np.uint32)
        h, w = self.pixels.shape
        if pack_order:
            self.handle = lib.refh_texture_create_ordered(_ptr(self.pixels), w, h, resolutions, pack_order)
        else:
            self.handle = lib.refh_texture_create(_ptr(self.pixels), w, h, resolutions)

    def info(self):
        fields = np.zeros(9, np.uint32)
        n = self.lib.refh_texture_info(self.handle, _ptr(fields), None, 0)
        pixels = np.zeros(n, np.uint32)
        self.lib.refh_texture_info(self.handle, _ptr(fields), _ptr(pixels), n)
        return fields, pixels

    def __del__(self):
        if _shut_down:
            return
        try:
            self.lib.refh_texture_free(self.handle)
        except Exception:
            pass


class RefModel:
    def __init__(self, scene, variant: str = "exact"):
        self.lib = _load(variant)
        self.scene = scene
        self.positions = np.ascontiguousarray(scene.positions, np.float32)
        self.poly = np.ascontiguousarray(scene.poly_indices, np.int32)
        self.tex = np.ascontiguousarray(scene.tex_coords, np.float32)
        self.colors = np.ascontiguousarray(scene.colors, np.float32)
        self.diffuse = RefTexture(self.lib, scene.diffuse, scene.diffuse_levels) if scene.diffuse is not None else None
        self.light = RefTexture(self.lib, scene.light, scene.light_levels) if scene.light is not None else None
        self.handle = self.lib.refh_model_create(
            _ptr(self.positions), self.positions.shape[0], _ptr(self.poly), _ptr(self.tex), _ptr(self.colors),
            self.poly.shape[0], self.diffuse.handle if self.diffuse else None,
            self.light.handle if self.light else None, scene.filter)
        self.camera = np.ascontiguousarray(scene.camera_location, np.float32)
        self.transform = np.ascontiguousarray(scene.model_to_world, np.float32)

    def __del__(self):
        if _shut_down:
            return
        try:
            self.lib.refh_model_free(self.handle)
        except Exception:
            pass

    def render(self, color=None, depth=None, *, pack_order: int = 0, threaded: bool = False,
               use_color: bool = True, use_depth: bool = True):
        s = self.scene
        h, w = s.height, s.width
        color = (np.zeros((h, w), np.uint32) if color is None else np.ascontiguousarray(color, np.uint32).copy()) if use_color else None
        depth = (np.zeros((h, w), np.float32) if depth is None else np.ascontiguousarray(depth, np.float32).copy()) if use_depth else None
        self.lib.refh_model_render(self.handle, _ptr(self.transform), _ptr(self.camera), int(s.perspective), s.slope,
                                   s.near_clip, s.far_clip, w, h, _ptr(color), _ptr(depth), pack_order, 1 if threaded else 0)
        return color, depth

    def render_depth(self, depth=None):
        s = self.scene
        depth = np.zeros((s.height, s.width), np.float32) if depth is None else np.ascontiguousarray(depth, np.float32).copy()
        self.lib.refh_model_render_depth(self.handle, _ptr(self.transform), _ptr(self.camera), int(s.perspective), s.slope,
                                         s.near_clip, s.far_clip, s.width, s.height, _ptr(depth))
        return depth


def triangle_rows(flat, clip, variant: str = "exact", max_rows: int = 1 << 16):
    l = _load(variant)
    flat = np.ascontiguousarray(flat, np.int64)
    clip = np.ascontiguousarray(clip, np.int32)
    start = np.zeros(1, np.int32)
    lefts = np.zeros(max_rows, np.int32)
    rights = np.zeros(max_rows, np.int32)
    n = l.refh_triangle_rows(_ptr(flat), _ptr(clip), 2, 2, _ptr(start), _ptr(lefts), _ptr(rights), max_rows)
    if n <= 0:
        return int(start[0]), lefts[:0], rights[:0]
    return int(start[0]), lefts[:n].copy(), rights[:n].copy()


# ---- deferred light passes and draw_higher through the reference's own functions

def _light_lib(variant: str):
    l = _load(variant)
    if not getattr(l, "_light_ready", False):
        P, I, F = C.c_void_p, C.c_int, C.c_float
        l.refh_ortho_view.argtypes = [F, I, I, P, P]
        l.refh_thread_count.restype = I
        l.refh_shadow_side.argtypes = [P, I, P]
        l.refh_directed_light.argtypes = [F, I, I, P, P, I, I, P, F, P, I]
        l.refh_point_light.argtypes = [F, I, I, I, I, P, P, P, I, I, P, F, F, P, P, I]
        l.refh_blend_light.argtypes = [P, I, P, P, I, I]
        l.refh_draw_higher.argtypes = [P, P, I, P, I, I, I, P, P, I, P, I, I, I, I, I, F]
        l.refh_dense_render.argtypes = [P, I, P, P, I, F, I, I, P, P, P, I, I, F, F, P, I]
        l.refh_light_frame.argtypes = [F, I, I, I, I, I, I, F, I, P, P, P, P, I, P, P, I, P, P, I, P, P, I, P, P, P, P]
        l.refh_light_frame.restype = C.c_double
        l._light_ready = True
    return l


def ortho_view(tilt: float, pixels_per_tile: int, index: int, variant: str = "exact"):
    l = _light_lib(variant)
    m = np.zeros(27, np.float32)
    i = np.zeros(5, np.int32)
    l.refh_ortho_view(tilt, pixels_per_tile, index, _ptr(m), _ptr(i))
    return m, i


def thread_count(variant: str = "exact") -> int:
    return int(_light_lib(variant).refh_thread_count())


def shadow_side(normal_to_world, side: int, variant: str = "exact"):
    out = np.zeros(12, np.float32)
    normal_to_world = np.ascontiguousarray(normal_to_world, np.float32)
    _light_lib(variant).refh_shadow_side(_ptr(normal_to_world), side, _ptr(out))
    return out


def directed_light(view, light, normal, direction, intensity, color, add, variant: str = "exact"):
    tilt, ppt, index = view
    light = np.ascontiguousarray(light, np.uint32).copy()
    normal = np.ascontiguousarray(normal, np.uint32)
    h, w = light.shape
    direction = np.asarray(direction, np.float32)  # kept alive across the call
    color = np.asarray(color, np.int32)
    _light_lib(variant).refh_directed_light(tilt, ppt, index, _ptr(light), _ptr(normal), w, h, _ptr(direction), intensity,
                                            _ptr(color), 1 if add else 0)
    return light


def point_light(view, center, light, normal, height, position, radius, intensity, color, cube=None, variant: str = "exact"):
    tilt, ppt, index = view
    light = np.ascontiguousarray(light, np.uint32).copy()
    h, w = light.shape
    cube_arr = None if cube is None else np.ascontiguousarray(cube, np.float32)
    normal = np.ascontiguousarray(normal, np.uint32)
    height = np.ascontiguousarray(height, np.float32)
    position = np.asarray(position, np.float32)
    color = np.asarray(color, np.int32)
    _light_lib(variant).refh_point_light(tilt, ppt, index, int(center[0]), int(center[1]), _ptr(light), _ptr(normal), _ptr(height),
                                         w, h, _ptr(position), radius, intensity, _ptr(color), _ptr(cube_arr),
                                         0 if cube_arr is None else cube_arr.shape[1])
    return light


def blend_light(target_pack_order, diffuse, light, variant: str = "exact"):
    diffuse = np.ascontiguousarray(diffuse, np.uint32)
    h, w = diffuse.shape
    out = np.zeros((h, w), np.uint32)
    light = np.ascontiguousarray(light, np.uint32)
    _light_lib(variant).refh_blend_light(_ptr(out), target_pack_order, _ptr(diffuse), _ptr(light), w, h)
    return out


def draw_higher(target, source, left, top, offset, variant: str = "exact"):
    """target, source: (height F32, A RGBA, A pack order, B RGBA, B pack order); returns the new target arrays."""
    th, ta, tap, tb, tbp = target
    sh, sa, sap, sb, sbp = source
    th, ta, tb = (np.ascontiguousarray(a).copy() for a in (th, ta, tb))
    sh = np.ascontiguousarray(sh, np.float32)
    sa = np.ascontiguousarray(sa, np.uint32)
    sb = np.ascontiguousarray(sb, np.uint32)
    H, W = th.shape
    h, w = sh.shape
    _light_lib(variant).refh_draw_higher(_ptr(th), _ptr(ta), tap, _ptr(tb), tbp, W, H, _ptr(sh), _ptr(sa), sap, _ptr(sb), sbp,
                                         w, h, left, top, offset)
    return th, ta, tb


def light_frame(scene, frames: int = 1, background_height: float = -1000.0, variant: str = "exact"):
    """One frame of the deferred-light pass (scenes.light_scene) through the reference's own
    functions (refh_light_frame): returns (seconds of the fastest of `frames` runs, output, light,
    height, cubes)."""
    l = _light_lib(variant)
    caster = RefModel(scene.caster, variant)
    sources = [(np.ascontiguousarray(h, np.float32), np.ascontiguousarray(c, np.uint32), np.ascontiguousarray(n, np.uint32))
               for h, c, n in zip(scene.sprite_heights, scene.sprite_diffuse, scene.sprite_normals)]
    types = np.array([[h.shape[1], h.shape[0]] for h, _, _ in sources], np.int32)
    ptrs = [(C.c_void_p * len(sources))(*[_ptr(s[k]) for s in sources]) for k in range(3)]
    placements = np.ascontiguousarray(scene.placements, np.int32)
    sun = np.array([*scene.sun_direction, scene.sun_intensity], np.float32)
    sun_color = np.array(scene.sun_color, np.int32)
    lights = np.array([[*x["position"], x["radius"], x["intensity"]] for x in scene.lights], np.float32).reshape(-1, 5)
    colors = np.array([x["color"] for x in scene.lights], np.int32).reshape(-1, 3)
    H, W, res = scene.height, scene.width, scene.cube_resolution
    output = np.zeros((H, W), np.uint32)
    light = np.zeros((H, W), np.uint32)
    height = np.zeros((H, W), np.float32)
    cubes = np.zeros((len(scene.lights), 6 * res, res), np.float32)
    seconds = l.refh_light_frame(scene.camera_tilt, scene.pixels_per_tile, scene.view_index, W, H, int(scene.center[0]),
                                 int(scene.center[1]), background_height, len(sources), _ptr(types), ptrs[0], ptrs[1], ptrs[2],
                                 len(placements), _ptr(placements), caster.handle, res, _ptr(sun), _ptr(sun_color), len(lights),
                                 _ptr(lights), _ptr(colors), frames, _ptr(output), _ptr(light), _ptr(height), _ptr(cubes))
    return float(seconds), output, light, height, list(cubes)


def dense_render(positions, polygons, colors, tilt, pixels_per_tile, view_index, height, diffuse, normal, origin, model_to_world,
                 high_quality: bool, variant: str = "exact"):
    """DenseModel_create + renderDenseModel<high_quality> of the reference; returns (height, diffuse, normal)."""
    positions = np.ascontiguousarray(positions, np.float32)
    polygons = np.ascontiguousarray(polygons, np.int32)
    colors = np.ascontiguousarray(colors, np.float32)
    height = np.ascontiguousarray(height, np.float32).copy()
    diffuse = np.ascontiguousarray(diffuse, np.uint32).copy()
    normal = np.ascontiguousarray(normal, np.uint32).copy()
    t = np.ascontiguousarray(model_to_world, np.float32)
    h, w = height.shape
    _light_lib(variant).refh_dense_render(_ptr(positions), len(positions), _ptr(polygons), _ptr(colors), len(polygons), tilt,
                                          pixels_per_tile, view_index, _ptr(height), _ptr(diffuse), _ptr(normal), w, h,
                                          origin[0], origin[1], _ptr(t), 1 if high_quality else 0)
    return height, diffuse, normal


def _camera_args(cam):
    """(location, perspective, slope, near, far, width, height) from a port.CameraDesc."""
    loc = np.array([cam.location[i] for i in range(12)], np.float32)
    return loc, [_ptr(loc), int(cam.perspective), float(cam.slope), float(cam.nearClip), float(cam.farClip),
                 int(cam.width), int(cam.height)]


class RefRenderer:
    """The reference's renderer_* with its occlusion grid; models are RefModel objects and cameras
    port.CameraDesc structures."""

    def __init__(self, variant: str = "exact"):
        self.lib = _load(variant)
        self.h = self.lib.refh_renderer_create()

    def __del__(self):
        if _shut_down:
            return
        try:
            self.lib.refh_renderer_free(self.h)
        except Exception:
            pass

    def begin(self, color, depth, pack_order: int = 0):
        img = color if color is not None else depth
        h, w = img.shape
        self.color = None if color is None else np.ascontiguousarray(color, np.uint32).copy()
        self.depth = None if depth is None else np.ascontiguousarray(depth, np.float32).copy()
        self.lib.refh_renderer_begin(self.h, _ptr(self.color), _ptr(self.depth), w, h, pack_order)

    def give_task(self, model: "RefModel", transform, cam):
        t = np.ascontiguousarray(transform, np.float32)
        loc, args = _camera_args(cam)
        self.lib.refh_renderer_give_task(self.h, model.handle, _ptr(t), *args)

    def occlude_from_box(self, mn, mx, transform, cam, debug_silhouette: bool = False):
        a, b = np.asarray(mn, np.float32), np.asarray(mx, np.float32)
        t = np.ascontiguousarray(transform, np.float32)
        loc, args = _camera_args(cam)
        self.lib.refh_renderer_occlude_from_box(self.h, _ptr(a), _ptr(b), _ptr(t), *args, 1 if debug_silhouette else 0)

    def occlude_from_existing_triangles(self):
        self.lib.refh_renderer_occlude_from_existing_triangles(self.h)

    def give_triangles(self, cs, is_, flat, colors, tex, diffuse: Optional["RefTexture"], light: Optional["RefTexture"],
                       filter_: int, cam):
        arrays = [np.ascontiguousarray(a, dt) for a, dt in ((cs, np.float32), (is_, np.float32), (flat, np.int64),
                                                              (colors, np.float32), (tex, np.float32))]
        loc, args = _camera_args(cam)
        for i in range(arrays[0].shape[0]):
            self.lib.refh_renderer_give_triangle(self.h, *[_ptr(a[i]) for a in arrays], diffuse.handle if diffuse else None,
                                                 light.handle if light else None, filter_, *args)

    def occlude_from_top_rows(self, cam):
        loc, args = _camera_args(cam)
        self.lib.refh_renderer_occlude_from_top_rows(self.h, *args)

    def is_box_visible(self, mn, mx, transform, cam) -> bool:
        a, b = np.asarray(mn, np.float32), np.asarray(mx, np.float32)
        t = np.ascontiguousarray(transform, np.float32)
        loc, args = _camera_args(cam)
        return bool(self.lib.refh_renderer_is_box_visible(self.h, _ptr(a), _ptr(b), _ptr(t), *args))

    def has_occluders(self) -> bool:
        return bool(self.lib.refh_renderer_has_occluders(self.h))

    def end(self, debug_wireframe: bool = False):
        self.lib.refh_renderer_end(self.h, 1 if debug_wireframe else 0)
        return self.color, self.depth


def draw_line(image, x1: int, y1: int, x2: int, y2: int, color: int, variant: str = "exact"):
    out = np.ascontiguousarray(image, np.uint32).copy()
    h, w = out.shape
    _load(variant).refh_draw_line(_ptr(out), w, h, x1, y1, x2, y2, color)
    return out
