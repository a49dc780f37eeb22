"""ctypes front end of the C oracle (oracle/dsr_oracle.c) -- test infrastructure only."""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")


def build(force: bool = False) -> str:
    src = os.path.join(HERE, "dsr_oracle.c")
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(src):
        subprocess.check_call(["gcc", "-std=c11", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-pthread",
                               src, "-o", LIB_PATH, "-lm"])
    return LIB_PATH


class Texture(C.Structure):
    _fields_ = [("log2width", C.c_uint32), ("log2height", C.c_uint32), ("maxMipLevel", C.c_uint32),
                ("startOffset", C.c_uint32), ("maxLevelMask", C.c_uint32),
                ("minWidthOrMask", C.c_uint32), ("minHeightOrMask", C.c_uint32),
                ("maxWidthAndMask", C.c_uint32), ("maxHeightAndMask", C.c_uint32),
                ("floatMaxWidth", C.c_float), ("floatMaxHeight", C.c_float),
                ("pixelCount", C.c_uint32), ("pixels", C.POINTER(C.c_uint32))]

    def array(self) -> np.ndarray:
        return np.ctypeslib.as_array(self.pixels, shape=(self.pixelCount,)).copy()

    def fields(self):
        return [self.log2width, self.log2height, self.maxMipLevel, self.startOffset, self.maxLevelMask,
                self.minWidthOrMask, self.minHeightOrMask, self.maxWidthAndMask, self.maxHeightAndMask]


class Model(C.Structure):
    _fields_ = [("positions", C.c_void_p), ("pointCount", C.c_int32), ("polyIndices", C.c_void_p),
                ("texCoords", C.c_void_p), ("colors", C.c_void_p), ("polyCount", C.c_int32),
                ("diffuse", C.POINTER(Texture)), ("light", C.POINTER(Texture)), ("filter", C.c_int32)]


class CameraDesc(C.Structure):
    _fields_ = [("location", C.c_float * 12), ("perspective", C.c_int32), ("slope", C.c_float),
                ("nearClip", C.c_float), ("farClip", C.c_float), ("width", C.c_int32), ("height", C.c_int32)]


class Stats(C.Structure):
    _fields_ = [("fragments", C.c_uint64), ("trianglesDrawn", C.c_uint64),
                ("coverage", C.c_void_p), ("winner", C.c_void_p)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        path = build()
        l = C.CDLL(path)
        P = C.c_void_p
        l.or_texture_init_empty.argtypes = [C.POINTER(Texture), C.c_uint32, C.c_uint32, C.c_uint32]
        l.or_texture_create_from_image.argtypes = [C.POINTER(Texture), P, C.c_int32, C.c_int32, C.c_int32]
        l.or_texture_create_from_image_ordered.argtypes = [C.POINTER(Texture), P, C.c_int32, C.c_int32, C.c_int32, C.c_int32]
        l.or_texture_free.argtypes = [C.POINTER(Texture)]
        l.or_texture_generate_pyramid.argtypes = [C.POINTER(Texture)]
        for name in ("or_texture_pixel_offset_to_layer",):
            getattr(l, name).argtypes = [C.POINTER(Texture), C.c_uint32]
            getattr(l, name).restype = C.c_uint32
        for name in ("or_texture_pixel_offset", "or_texture_read_pixel"):
            getattr(l, name).argtypes = [C.POINTER(Texture), C.c_uint32, C.c_uint32, C.c_uint32]
            getattr(l, name).restype = C.c_uint32
        l.or_texture_write_pixel.argtypes = [C.POINTER(Texture), C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32]
        l.or_interpolate_color_linear.argtypes = [C.c_uint32] * 3
        l.or_interpolate_color_linear.restype = C.c_uint32
        l.or_interpolate_color_bilinear.argtypes = [C.c_uint32] * 6
        l.or_interpolate_color_bilinear.restype = C.c_uint32
        l.or_sample_bilinear.argtypes = [C.POINTER(Texture), C.c_float, C.c_float, C.c_uint32, C.c_int]
        l.or_sample_bilinear.restype = C.c_uint32
        l.or_sample_nearest.argtypes = [C.POINTER(Texture), C.c_float, C.c_float, C.c_uint32, C.c_int]
        l.or_sample_nearest.restype = C.c_uint32
        l.or_camera_to_screen.argtypes = [C.POINTER(CameraDesc), P, P, P]
        l.or_triangle_rows.argtypes = [P, P, P, P, P, C.c_int32]
        l.or_triangle_rows.restype = C.c_int32
        l.or_model_render.argtypes = [C.POINTER(Model), P, C.POINTER(CameraDesc), P, P, C.c_int32, C.c_int32,
                                      C.c_int32, C.POINTER(Stats)]
        l.or_model_render.restype = C.c_int
        l.or_model_render_depth.argtypes = [C.POINTER(Model), P, C.POINTER(CameraDesc), P, C.POINTER(Stats)]
        l.or_model_render_depth.restype = C.c_int
        R = C.c_void_p
        l.or_renderer_create.restype = R
        l.or_renderer_destroy.argtypes = [R]
        l.or_renderer_begin.argtypes = [R, P, P, C.c_int32, C.c_int32, C.c_int32]
        l.or_renderer_give_task.argtypes = [R, C.POINTER(Model), P, C.POINTER(CameraDesc)]
        l.or_renderer_occlude_from_box.argtypes = [R, P, P, P, C.POINTER(CameraDesc), C.c_int]
        l.or_renderer_occlude_from_existing_triangles.argtypes = [R]
        l.or_renderer_give_triangle.argtypes = [R, P, P, P, P, P, C.POINTER(Texture), C.POINTER(Texture), C.c_int,
                                                C.POINTER(CameraDesc)]
        l.or_world_to_screen.argtypes = [C.POINTER(CameraDesc), P, P, P]
        l.or_renderer_occlude_from_top_rows.argtypes = [R, C.c_int]
        l.or_renderer_is_box_visible.argtypes = [R, P, P, P, C.POINTER(CameraDesc)]
        l.or_renderer_has_occluders.argtypes = [R]
        l.or_renderer_end.argtypes = [R, C.POINTER(Stats), C.c_int]
        l.or_draw_line.argtypes = [P, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_uint32]
        l.or_renderer_grid.argtypes = [R, P, P, P]
        _lib = l
    return _lib


def _ptr(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class OracleTexture:
    def __init__(self, pixels: Optional[np.ndarray] = None, resolutions: int = 16, empty=None, pack_order: int = 0):
        self.t = Texture()
        if empty is not None:
            if lib().or_texture_init_empty(C.byref(self.t), *empty):
                raise MemoryError
        else:
            pixels = np.ascontiguousarray(pixels, dtype=np.uint32)
            h, w = pixels.shape
            if lib().or_texture_create_from_image_ordered(C.byref(self.t), _ptr(pixels), w, h, resolutions, pack_order):
                raise ValueError("texture dimensions must be powers of two")

    def __del__(self):
        try:
            lib().or_texture_free(C.byref(self.t))
        except Exception:
            pass

    def ref(self):
        return C.pointer(self.t)


def camera_desc(scene) -> CameraDesc:
    d = CameraDesc()
    for i in range(12):
        d.location[i] = float(scene.camera_location[i])
    d.perspective = 1 if scene.perspective else 0
    d.slope = scene.slope
    d.nearClip = scene.near_clip
    d.farClip = scene.far_clip
    d.width = scene.width
    d.height = scene.height
    return d


class PreparedModel:
    """Keeps the numpy buffers and textures of one scene alive for repeated renders."""

    def __init__(self, scene):
        self.scene = scene
        self.positions = np.ascontiguousarray(scene.positions, np.float32)
        self.poly = np.ascontiguousarray(scene.poly_indices, np.int32)
        self.tex = np.ascontiguousarray(scene.tex_coords, np.float32)
        self.colors = np.ascontiguousarray(scene.colors, np.float32)
        self.diffuse = OracleTexture(scene.diffuse, scene.diffuse_levels) if scene.diffuse is not None else None
        self.light = OracleTexture(scene.light, scene.light_levels) if scene.light is not None else None
        m = Model()
        m.positions = _ptr(self.positions)
        m.pointCount = self.positions.shape[0]
        m.polyIndices = _ptr(self.poly)
        m.texCoords = _ptr(self.tex)
        m.colors = _ptr(self.colors)
        m.polyCount = self.poly.shape[0]
        m.diffuse = self.diffuse.ref() if self.diffuse else None
        m.light = self.light.ref() if self.light else None
        m.filter = scene.filter
        self.model = m
        self.cam = camera_desc(scene)
        self.transform = np.ascontiguousarray(scene.model_to_world, np.float32)


def render(scene, color: Optional[np.ndarray] = None, depth: Optional[np.ndarray] = None, *, pack_order: int = 0,
           bands: int = 1, threads: int = 1, use_color: bool = True, use_depth: bool = True,
           coverage: bool = False, winner: bool = False, prepared: Optional[PreparedModel] = None):
    """model_render (bands == 1) or the band-split renderer (bands > 1) on the CPU oracle.

    Returns (color, depth, info) where info holds fragments, trianglesDrawn and the optional
    per-pixel coverage counts and winner keys."""
    pm = prepared or PreparedModel(scene)
    h, w = scene.height, scene.width
    if use_color:
        color = np.zeros((h, w), np.uint32) if color is None else np.ascontiguousarray(color, np.uint32).copy()
    else:
        color = None
    if use_depth:
        depth = np.zeros((h, w), np.float32) if depth is None else np.ascontiguousarray(depth, np.float32).copy()
    else:
        depth = None
    st = Stats()
    cov = np.zeros((h, w), np.uint32) if coverage else None
    win = np.full((h, w), 0xFFFFFFFF, np.uint32) if winner else None
    st.coverage = _ptr(cov)
    st.winner = _ptr(win)
    lib().or_model_render(C.byref(pm.model), _ptr(pm.transform), C.byref(pm.cam), _ptr(color), _ptr(depth),
                          pack_order, bands, threads, C.byref(st))
    info = {"fragments": int(st.fragments), "triangles_drawn": int(st.trianglesDrawn), "coverage": cov, "winner": win}
    return color, depth, info


def render_depth(scene, depth: Optional[np.ndarray] = None, *, coverage: bool = False, winner: bool = False,
                 prepared: Optional[PreparedModel] = None):
    pm = prepared or PreparedModel(scene)
    h, w = scene.height, scene.width
    depth = np.zeros((h, w), np.float32) if depth is None else np.ascontiguousarray(depth, np.float32).copy()
    st = Stats()
    cov = np.zeros((h, w), np.uint32) if coverage else None
    win = np.full((h, w), 0xFFFFFFFF, np.uint32) if winner else None
    st.coverage = _ptr(cov)
    st.winner = _ptr(win)
    lib().or_model_render_depth(C.byref(pm.model), _ptr(pm.transform), C.byref(pm.cam), _ptr(depth), C.byref(st))
    return depth, {"fragments": int(st.fragments), "triangles_drawn": int(st.trianglesDrawn), "coverage": cov,
                   "winner": win}


def triangle_rows(flat, clip, max_rows: int = 1 << 16):
    flat = np.ascontiguousarray(flat, np.int64)
    clip = np.ascontiguousarray(clip, np.int32)
    start = np.zeros(1, np.int32)
    lefts = np.zeros(max_rows, np.int32)
    rights = np.zeros(max_rows, np.int32)
    n = lib().or_triangle_rows(_ptr(flat), _ptr(clip), _ptr(start), _ptr(lefts), _ptr(rights), max_rows)
    if n <= 0:
        return int(start[0]), lefts[:0], rights[:0]
    return int(start[0]), lefts[:n].copy(), rights[:n].copy()


def camera_to_screen(scene, cs):
    d = camera_desc(scene)
    cs = np.ascontiguousarray(cs, np.float32)
    out_is = np.zeros(2, np.float32)
    out_flat = np.zeros(2, np.int64)
    lib().or_camera_to_screen(C.byref(d), _ptr(cs), _ptr(out_is), _ptr(out_flat))
    return out_is, out_flat


# ---- deferred light passes and draw_higher (oracle/dsr_oracle.c)

class OrthoView(C.Structure):
    _fields_ = [("normalToWorld", C.c_float * 9), ("screenDepthToLightSpace", C.c_float * 9),
                ("lightSpaceToScreenDepth", C.c_float * 9), ("pixelOffsetPerTileX", C.c_int32 * 2),
                ("pixelOffsetPerTileZ", C.c_int32 * 2), ("yPixelsPerTile", C.c_int32)]

    def arrays(self):
        m = np.concatenate([np.ctypeslib.as_array(self.normalToWorld), np.ctypeslib.as_array(self.screenDepthToLightSpace),
                            np.ctypeslib.as_array(self.lightSpaceToScreenDepth)]).astype(np.float32)
        i = np.array([*self.pixelOffsetPerTileX, *self.pixelOffsetPerTileZ, self.yPixelsPerTile], np.int32)
        return m, i


def _light_lib():
    l = lib()
    if not getattr(l, "_light_ready", False):
        P, I, F = C.c_void_p, C.c_int32, C.c_float
        l.or_ortho_view_create.argtypes = [F, I, I, C.POINTER(OrthoView)]
        l.or_dense_triangle_count.argtypes = [P, I]
        l.or_dense_triangle_count.restype = I
        l.or_dense_model_create.argtypes = [P, I, P, P, I, P]
        l.or_dense_render.argtypes = [P, I, C.POINTER(OrthoView), P, I, P, I, P, I, I, I, F, F, P, I]
        l.or_shadow_side_location.argtypes = [P, I, P]
        l.or_directed_light.argtypes = [C.POINTER(OrthoView), P, I, P, I, I, I, P, F, P, I]
        l.or_point_light_bound.argtypes = [C.POINTER(OrthoView), I, I, I, I, P, F, P]
        l.or_point_light_bound.restype = I
        l.or_point_light.argtypes = [C.POINTER(OrthoView), I, I, P, I, P, I, P, I, I, I, P, F, F, P, P, I, I]
        l.or_blend_light.argtypes = [P, I, I, P, I, P, I, I, I]
        l.or_draw_higher.argtypes = [P, I, P, I, I, P, I, I, I, I, P, I, P, I, I, P, I, I, I, I, I, I, F]
        l._light_ready = True
    return l


def ortho_view(tilt: float, pixels_per_tile: int, index: int) -> OrthoView:
    v = OrthoView()
    _light_lib().or_ortho_view_create(tilt, pixels_per_tile, index, C.byref(v))
    return v


def shadow_side(normal_to_world, side: int):
    out = np.zeros(12, np.float32)
    normal_to_world = np.ascontiguousarray(normal_to_world, np.float32)
    _light_lib().or_shadow_side_location(normal_to_world.ctypes.data, side, out.ctypes.data)
    return out


def directed_light(view: OrthoView, light, normal, direction, intensity, color, add):
    light = np.ascontiguousarray(light, np.uint32).copy()
    normal = np.ascontiguousarray(normal, np.uint32)
    h, w = light.shape
    direction = np.asarray(direction, np.float32)  # kept alive across the call
    color = np.asarray(color, np.int32)
    _light_lib().or_directed_light(C.byref(view), light.ctypes.data, w, normal.ctypes.data, w, w, h,
                                   direction.ctypes.data, intensity, color.ctypes.data, 1 if add else 0)
    return light


def point_light_bound(view: OrthoView, center, width, height, position, radius):
    b = np.zeros(4, np.int32)
    position = np.asarray(position, np.float32)
    ok = _light_lib().or_point_light_bound(C.byref(view), int(center[0]), int(center[1]), width, height,
                                           position.ctypes.data, radius, b.ctypes.data)
    return b if ok else None


def point_light(view: OrthoView, center, light, normal, height, position, radius, intensity, color, cube=None, threads=1):
    light = np.ascontiguousarray(light, np.uint32).copy()
    normal = np.ascontiguousarray(normal, np.uint32)
    height = np.ascontiguousarray(height, np.float32)
    h, w = light.shape
    cube_arr = None if cube is None else np.ascontiguousarray(cube, np.float32)
    position = np.asarray(position, np.float32)
    color = np.asarray(color, np.int32)
    _light_lib().or_point_light(C.byref(view), int(center[0]), int(center[1]), light.ctypes.data, w, normal.ctypes.data, w,
                                height.ctypes.data, w, w, h, position.ctypes.data, radius, intensity, color.ctypes.data,
                                None if cube_arr is None else cube_arr.ctypes.data, 0 if cube_arr is None else cube_arr.shape[1],
                                threads)
    return light


def blend_light(target_pack_order, diffuse, light):
    diffuse = np.ascontiguousarray(diffuse, np.uint32)
    light = np.ascontiguousarray(light, np.uint32)
    h, w = diffuse.shape
    out = np.zeros((h, w), np.uint32)
    _light_lib().or_blend_light(out.ctypes.data, w, target_pack_order, diffuse.ctypes.data, w, light.ctypes.data, w, w, h)
    return out


def draw_higher(target, source, left, top, offset):
    th, ta, tap, tb, tbp = target
    th = np.ascontiguousarray(th, np.float32).copy()
    ta = np.ascontiguousarray(ta, np.uint32).copy()
    tb = np.ascontiguousarray(tb, np.uint32).copy()
    draw_higher_in_place((th, ta, tap, tb, tbp), source, left, top, offset)
    return th, ta, tb


def draw_higher_in_place(target, source, left, top, offset):
    """draw_higher into target images that are C-contiguous float32 / uint32 arrays, changed in place."""
    th, ta, tap, tb, tbp = target
    sh, sa, sap, sb, sbp = source
    assert th.flags.c_contiguous and ta.flags.c_contiguous and tb.flags.c_contiguous
    assert th.dtype == np.float32 and ta.dtype == np.uint32 and tb.dtype == np.uint32
    sh = np.ascontiguousarray(sh, np.float32)
    sa = np.ascontiguousarray(sa, np.uint32)
    sb = np.ascontiguousarray(sb, np.uint32)
    H, W = th.shape
    h, w = sh.shape
    _light_lib().or_draw_higher(th.ctypes.data, W, ta.ctypes.data, W, tap, tb.ctypes.data, W, tbp, W, H, sh.ctypes.data, w,
                                sa.ctypes.data, w, sap, sb.ctypes.data, w, sbp, w, h, left, top, offset)


class OracleRenderer:
    """renderer_begin / giveTask / the occlusion grid / renderer_end on the CPU oracle
    (api/rendererAPI.cpp:141-477).  Models are PreparedModel objects; cameras CameraDesc."""

    def __init__(self):
        self.h = C.c_void_p(lib().or_renderer_create())
        self._keep = []

    def __del__(self):
        try:
            lib().or_renderer_destroy(self.h)
        except Exception:
            pass

    def begin(self, color: Optional[np.ndarray], depth: Optional[np.ndarray], pack_order: int = 0):
        img = color if color is not None else depth
        h, w = img.shape
        self.color = None if color is None else np.ascontiguousarray(color, np.uint32).copy()
        self.depth = None if depth is None else np.ascontiguousarray(depth, np.float32).copy()
        self._keep = []
        assert lib().or_renderer_begin(self.h, _ptr(self.color), _ptr(self.depth), w, h, pack_order) == 0

    def give_task(self, pm: "PreparedModel", transform=None, cam: Optional[CameraDesc] = None):
        t = np.ascontiguousarray(pm.transform if transform is None else transform, np.float32)
        self._keep.append((pm, t))
        assert lib().or_renderer_give_task(self.h, C.byref(pm.model), _ptr(t), C.byref(cam or pm.cam)) == 0

    def occlude_from_box(self, mn, mx, transform, cam: CameraDesc, debug_silhouette: bool = False):
        a, b = np.asarray(mn, np.float32), np.asarray(mx, np.float32)
        t = np.ascontiguousarray(transform, np.float32)
        assert lib().or_renderer_occlude_from_box(self.h, _ptr(a), _ptr(b), _ptr(t), C.byref(cam), 1 if debug_silhouette else 0) == 0

    def occlude_from_existing_triangles(self):
        assert lib().or_renderer_occlude_from_existing_triangles(self.h) == 0

    def give_triangles(self, cs, is_, flat, colors, tex, diffuse: Optional["OracleTexture"], light: Optional["OracleTexture"],
                       filter_: int, cam: CameraDesc):
        """cs (n, 3, 3) float32, is_ (n, 3, 2) float32, flat (n, 3, 2) int64, colors and tex (n, 3, 4) float32."""
        arrays = [np.ascontiguousarray(a, dt) for a, dt in ((cs, np.float32), (is_, np.float32), (flat, np.int64),
                                                              (colors, np.float32), (tex, np.float32))]
        self._keep.append((arrays, diffuse, light))
        n = arrays[0].shape[0]
        for i in range(n):
            assert lib().or_renderer_give_triangle(self.h, *[_ptr(a[i]) for a in arrays], diffuse.ref() if diffuse else None,
                                                   light.ref() if light else None, filter_, C.byref(cam)) == 0

    def occlude_from_top_rows(self, perspective: bool):
        return lib().or_renderer_occlude_from_top_rows(self.h, 1 if perspective else 0)

    def is_box_visible(self, mn, mx, transform, cam: CameraDesc) -> bool:
        a, b = np.asarray(mn, np.float32), np.asarray(mx, np.float32)
        t = np.ascontiguousarray(transform, np.float32)
        return bool(lib().or_renderer_is_box_visible(self.h, _ptr(a), _ptr(b), _ptr(t), C.byref(cam)))

    def has_occluders(self) -> bool:
        return bool(lib().or_renderer_has_occluders(self.h))

    def grid(self):
        gw, gh = C.c_int32(0), C.c_int32(0)
        lib().or_renderer_grid(self.h, None, C.cast(C.pointer(gw), C.c_void_p), C.cast(C.pointer(gh), C.c_void_p))
        out = np.zeros((gh.value, gw.value), np.float32)
        lib().or_renderer_grid(self.h, _ptr(out), C.cast(C.pointer(gw), C.c_void_p), C.cast(C.pointer(gh), C.c_void_p))
        return out

    def end(self, coverage: bool = False, debug_wireframe: bool = False):
        st = Stats()
        cov = None
        if coverage:
            img = self.color if self.color is not None else self.depth
            cov = np.zeros(img.shape, np.uint32)
        st.coverage = _ptr(cov)
        assert lib().or_renderer_end(self.h, C.byref(st), 1 if debug_wireframe else 0) == 0
        return self.color, self.depth, {"fragments": int(st.fragments), "coverage": cov}


def draw_line(image: np.ndarray, x1: int, y1: int, x2: int, y2: int, color: int) -> np.ndarray:
    out = np.ascontiguousarray(image, np.uint32).copy()
    h, w = out.shape
    lib().or_draw_line(_ptr(out), w, h, x1, y1, x2, y2, color)
    return out


def world_to_screen(cam: CameraDesc, world) -> tuple:
    """Camera::worldToScreen of (n, 3) points: cs (n, 3), is (n, 2), flat (n, 2) int64."""
    world = np.ascontiguousarray(world, np.float32).reshape(-1, 3)
    out = np.zeros((len(world), 5), np.float32)
    flat = np.zeros((len(world), 2), np.int64)
    for i in range(len(world)):
        lib().or_world_to_screen(C.byref(cam), _ptr(world[i]), _ptr(out[i]), _ptr(flat[i]))
    return out[:, :3].copy(), out[:, 3:].copy(), flat


# ---- dense models of the sprite engine (SDK/SpriteEngine/spriteAPI.cpp:1174-1327)

DENSE_TRIANGLE = np.dtype([("color", np.float32, (3, 3)), ("pos", np.float32, (3, 3)), ("normal", np.float32, (3, 3))])


def dense_model(positions, polygons, colors) -> np.ndarray:
    """DenseModel_create: one dense triangle (colours x 255, corners, smooth normals) per fan triangle."""
    l = _light_lib()
    positions = np.ascontiguousarray(positions, np.float32)
    polygons = np.ascontiguousarray(polygons, np.int32)
    colors = np.ascontiguousarray(colors, np.float32)
    n = l.or_dense_triangle_count(polygons.ctypes.data, len(polygons))
    out = np.zeros(max(n, 1), DENSE_TRIANGLE)
    l.or_dense_model_create(positions.ctypes.data, len(positions), polygons.ctypes.data, colors.ctypes.data, len(polygons),
                            out.ctypes.data)
    return out[:n]


def dense_render(triangles, view: OrthoView, height, diffuse, normal, origin, model_to_world, high_quality: bool):
    """renderDenseModel<high_quality> into copies of the images; returns (height, diffuse, normal)."""
    l = _light_lib()
    triangles = np.ascontiguousarray(triangles, DENSE_TRIANGLE)
    height = np.ascontiguousarray(height, np.float32).copy()
    diffuse = np.ascontiguousarray(diffuse, np.uint32).copy()
    normal = np.ascontiguousarray(normal, np.uint32).copy()
    h, w = height.shape
    t = np.ascontiguousarray(model_to_world, np.float32)
    l.or_dense_render(triangles.ctypes.data if len(triangles) else None, len(triangles), C.byref(view), height.ctypes.data, w,
                      diffuse.ctypes.data, w, normal.ctypes.data, w, w, h, C.c_float(origin[0]), C.c_float(origin[1]),
                      t.ctypes.data, 1 if high_quality else 0)
    return height, diffuse, normal
