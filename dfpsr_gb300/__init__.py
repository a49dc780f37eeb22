"""GB300 (sm_103a) implementation of DFPSR's triangle-rendering path.

The product is the in-tree CUDA library libdsrg.so behind the C ABI in
include/dsrg.h.  This module is a thin ctypes front end over that ABI for Python
callers (tests, benchmarks, the gradient harness).  There is no fallback: if the
library is missing or no GPU is present, calls raise.
"""
from __future__ import annotations

import ctypes as C
import os
import weakref
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libdsrg.so")

DSRG_OK = 0
STATUS_NAMES = {0: "OK", 1: "INVALID_ARGUMENT", 2: "CUDA", 3: "OUT_OF_MEMORY", 4: "CALL_ORDER", 5: "UNSUPPORTED", 6: "DEVICE"}

# Every entry point declared in include/dsrg.h.
EXPORTED = [
    "dsrg_context_create", "dsrg_context_destroy", "dsrg_context_last_error", "dsrg_context_stream",
    "dsrg_context_set_counting", "dsrg_context_get_stats", "dsrg_context_walked_fragments", "dsrg_debug_fail_allocation",
    "dsrg_texture_create", "dsrg_texture_destroy", "dsrg_texture_read", "dsrg_texture_create_many", "dsrg_texture_upload",
    "dsrg_model_create", "dsrg_model_destroy", "dsrg_model_set_bound",
    "dsrg_model_render", "dsrg_model_render_depth",
    "dsrg_renderer_create", "dsrg_renderer_destroy", "dsrg_renderer_begin", "dsrg_renderer_give_task",
    "dsrg_renderer_end", "dsrg_renderer_takes_triangles", "dsrg_model_render_depth_noalloc",
    "dsrg_batch_create", "dsrg_batch_destroy", "dsrg_batch_clear", "dsrg_batch_add_frame", "dsrg_batch_give_task",
    "dsrg_batch_render", "dsrg_context_get_tuning", "dsrg_context_set_tuning", "dsrg_batch_autotune",
    "dsrg_diff_create", "dsrg_diff_destroy", "dsrg_diff_forward", "dsrg_diff_l2_loss", "dsrg_diff_adjoint",
    "dsrg_ortho_view_create", "dsrg_shadow_side_location", "dsrg_light_directed", "dsrg_light_points", "dsrg_light_blend",
    "dsrg_draw_higher", "dsrg_sprite_frame", "dsrg_check_float_roots", "dsrg_batch_set_depth_only", "dsrg_batch_set_tuning",
    "dsrg_dense_model_create", "dsrg_dense_model_destroy", "dsrg_dense_render", "dsrg_dense_render_many",
    "dsrg_renderer_occlude_from_box", "dsrg_renderer_occlude_from_existing_triangles", "dsrg_renderer_occlude_from_top_rows",
    "dsrg_renderer_is_box_visible", "dsrg_renderer_has_occluders", "dsrg_renderer_get_occlusion_grid",
    "dsrg_renderer_end_debug", "dsrg_renderer_get_images", "dsrg_camera_world_to_screen", "dsrg_renderer_give_triangles",
]


class DsrgError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status
        self.message = message


class Camera(C.Structure):
    _fields_ = [("location", C.c_float * 12), ("perspective", C.c_int32), ("slope", C.c_float),
                ("nearClip", C.c_float), ("farClip", C.c_float), ("width", C.c_int32), ("height", C.c_int32)]


class Image(C.Structure):
    _fields_ = [("data", C.c_void_p), ("width", C.c_int32), ("height", C.c_int32), ("strideBytes", C.c_int32),
                ("packOrder", C.c_int32), ("onDevice", C.c_int32)]


class Stats(C.Structure):
    _fields_ = [("fragments", C.c_uint64), ("drawRecords", C.c_uint64), ("binEntries", C.c_uint64),
                ("milliseconds", C.c_float), ("rasterMilliseconds", C.c_float), ("kernelLaunches", C.c_uint64)]


class Tuning(C.Structure):
    _fields_ = [("threadsPerTile", C.c_int32), ("ctasPerSm", C.c_int32), ("smallRows", C.c_int32),
                ("smallWidth", C.c_int32), ("graphs", C.c_int32), ("resolve", C.c_int32)]

    def as_dict(self) -> dict:
        return {"threads_per_tile": self.threadsPerTile, "ctas_per_sm": self.ctasPerSm, "small_rows": self.smallRows,
                "small_width": self.smallWidth, "graphs": self.graphs, "resolve": self.resolve}


class OrthoView(C.Structure):
    _fields_ = [("normalToWorld", C.c_float * 9), ("screenDepthToLightSpace", C.c_float * 9),
                ("lightSpaceToScreenDepth", C.c_float * 9), ("pixelOffsetPerTileX", C.c_int32 * 2),
                ("pixelOffsetPerTileZ", C.c_int32 * 2), ("yPixelsPerTile", C.c_int32)]

    def arrays(self):
        m = np.concatenate([np.ctypeslib.as_array(self.normalToWorld), np.ctypeslib.as_array(self.screenDepthToLightSpace),
                            np.ctypeslib.as_array(self.lightSpaceToScreenDepth)]).astype(np.float32)
        i = np.array([*self.pixelOffsetPerTileX, *self.pixelOffsetPerTileZ, self.yPixelsPerTile], np.int32)
        return m, i


class PointLight(C.Structure):
    _fields_ = [("position", C.c_float * 3), ("radius", C.c_float), ("intensity", C.c_float), ("color", C.c_int32 * 3),
                ("shadowCube", C.c_void_p), ("cubeWidth", C.c_int32)]


class Sprite(C.Structure):
    _fields_ = [("height", C.c_void_p), ("colorA", C.c_void_p), ("colorB", C.c_void_p), ("width", C.c_int32),
                ("height_", C.c_int32), ("heightStrideBytes", C.c_int32), ("colorAStrideBytes", C.c_int32),
                ("colorBStrideBytes", C.c_int32), ("colorAPackOrder", C.c_int32), ("colorBPackOrder", C.c_int32),
                ("left", C.c_int32), ("top", C.c_int32), ("offset", C.c_float), ("onDevice", C.c_int32)]


class SpriteFrame(C.Structure):
    """dsrg_sprite_frame_desc: one frame of the deferred-light pass."""
    _fields_ = [("view", C.POINTER(OrthoView)), ("centerX", C.c_int32), ("centerY", C.c_int32),
                ("height", C.POINTER(Image)), ("diffuse", C.POINTER(Image)), ("normal", C.POINTER(Image)),
                ("light", C.POINTER(Image)), ("output", C.POINTER(Image)), ("clearHeight", C.c_float),
                ("clearDiffuse", C.c_uint32), ("clearNormal", C.c_uint32), ("sprites", C.POINTER(Sprite)),
                ("spriteCount", C.c_int32), ("sunDirection", C.c_float * 3), ("sunIntensity", C.c_float),
                ("sunColor", C.c_int32 * 3), ("shadows", C.c_void_p), ("lights", C.POINTER(PointLight)),
                ("lightCount", C.c_int32), ("referenceThreads", C.c_int32)]


_lib = None


def lib():
    """Loads libdsrg.so (built by __graft_entry__.build() or dfpsr_gb300.build)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
        l = C.CDLL(LIB_PATH)
        P, I = C.c_void_p, C.c_int32
        l.dsrg_context_create.argtypes = [I, C.POINTER(P)]
        l.dsrg_context_destroy.argtypes = [P]
        l.dsrg_context_last_error.argtypes = [P]
        l.dsrg_context_last_error.restype = C.c_char_p
        l.dsrg_context_stream.argtypes = [P]
        l.dsrg_context_stream.restype = P
        l.dsrg_context_set_counting.argtypes = [P, I, P]
        l.dsrg_context_get_stats.argtypes = [P, C.POINTER(Stats)]
        l.dsrg_context_walked_fragments.argtypes = [P, C.POINTER(C.c_uint64)]
        l.dsrg_debug_fail_allocation.argtypes = [C.c_int64]
        l.dsrg_texture_create.argtypes = [P, P, I, I, I, C.POINTER(P)]
        l.dsrg_texture_destroy.argtypes = [P]
        l.dsrg_texture_read.argtypes = [P, P, I, P, C.POINTER(I)]
        l.dsrg_texture_create_many.argtypes = [P, I, C.POINTER(Image), P, C.POINTER(P)]
        l.dsrg_model_create.argtypes = [P, P, I, P, P, P, I, P, P, I, C.POINTER(P)]
        l.dsrg_model_destroy.argtypes = [P]
        l.dsrg_model_render.argtypes = [P, P, P, C.POINTER(Camera), C.POINTER(Image), C.POINTER(Image)]
        l.dsrg_model_render_depth.argtypes = [P, P, P, C.POINTER(Camera), C.POINTER(Image)]
        l.dsrg_renderer_create.argtypes = [P, C.POINTER(P)]
        l.dsrg_renderer_destroy.argtypes = [P]
        l.dsrg_renderer_begin.argtypes = [P, C.POINTER(Image), C.POINTER(Image)]
        l.dsrg_renderer_give_task.argtypes = [P, P, P, C.POINTER(Camera)]
        l.dsrg_renderer_end.argtypes = [P]
        l.dsrg_renderer_takes_triangles.argtypes = [P]
        l.dsrg_renderer_occlude_from_box.argtypes = [P, P, P, P, C.POINTER(Camera), I]
        l.dsrg_renderer_occlude_from_existing_triangles.argtypes = [P]
        l.dsrg_renderer_occlude_from_top_rows.argtypes = [P, C.POINTER(Camera)]
        l.dsrg_renderer_is_box_visible.argtypes = [P, P, P, P, C.POINTER(Camera), C.POINTER(I)]
        l.dsrg_renderer_has_occluders.argtypes = [P]
        l.dsrg_renderer_get_occlusion_grid.argtypes = [P, P, I, C.POINTER(I), C.POINTER(I)]
        l.dsrg_renderer_end_debug.argtypes = [P, I]
        l.dsrg_renderer_get_images.argtypes = [P, C.POINTER(Image), C.POINTER(Image)]
        l.dsrg_camera_world_to_screen.argtypes = [C.POINTER(Camera), P, P]
        l.dsrg_renderer_give_triangles.argtypes = [P, I, P, P, P, P, P, I, C.POINTER(Camera)]
        l.dsrg_model_render_depth_noalloc.argtypes = [P, P, P, C.POINTER(Camera), C.POINTER(Image)]
        l.dsrg_batch_create.argtypes = [P, C.POINTER(P)]
        l.dsrg_batch_destroy.argtypes = [P]
        l.dsrg_batch_clear.argtypes = [P]
        l.dsrg_batch_add_frame.argtypes = [P, C.POINTER(Image), C.POINTER(Image), C.POINTER(I)]
        l.dsrg_batch_give_task.argtypes = [P, I, P, P, C.POINTER(Camera)]
        l.dsrg_batch_render.argtypes = [P]
        l.dsrg_context_get_tuning.argtypes = [P, C.POINTER(Tuning)]
        l.dsrg_context_set_tuning.argtypes = [P, C.POINTER(Tuning)]
        l.dsrg_batch_autotune.argtypes = [P, I, C.POINTER(Tuning)]
        l.dsrg_diff_create.argtypes = [P, P, I, I, C.c_float, C.POINTER(P)]
        l.dsrg_diff_destroy.argtypes = [P]
        l.dsrg_diff_forward.argtypes = [P, I, C.POINTER(Camera), P, P, P, P, P, P]
        l.dsrg_diff_l2_loss.argtypes = [P, C.c_int64, P, P, P, P]
        l.dsrg_diff_adjoint.argtypes = [P, I, I, I, P, P, P, P, P, P, P, P, P, I]
        l.dsrg_ortho_view_create.argtypes = [C.c_float, I, I, C.POINTER(OrthoView)]
        l.dsrg_shadow_side_location.argtypes = [P, I, P]
        l.dsrg_light_directed.argtypes = [P, C.POINTER(OrthoView), C.POINTER(Image), C.POINTER(Image), P, C.c_float, P, I]
        l.dsrg_light_points.argtypes = [P, C.POINTER(OrthoView), I, I, C.POINTER(Image), C.POINTER(Image), C.POINTER(Image),
                                        C.POINTER(PointLight), I, I]
        l.dsrg_light_blend.argtypes = [P, C.POINTER(Image), C.POINTER(Image), C.POINTER(Image)]
        l.dsrg_draw_higher.argtypes = [P, C.POINTER(Image), C.POINTER(Image), C.POINTER(Image), C.POINTER(Sprite), I]
        l.dsrg_dense_model_create.argtypes = [P, P, I, P, P, I, C.POINTER(P)]
        l.dsrg_dense_model_destroy.argtypes = [P]
        l.dsrg_dense_render.argtypes = [P, P, C.POINTER(OrthoView), C.POINTER(Image), C.POINTER(Image), C.POINTER(Image),
                                        C.c_float, C.c_float, P, I]
        l.dsrg_dense_render_many.argtypes = [P, P, I, C.POINTER(OrthoView), C.POINTER(Image), C.POINTER(Image), C.POINTER(Image), I]
        l.dsrg_batch_set_depth_only.argtypes = [P, I]
        l.dsrg_batch_set_tuning.argtypes = [P, C.POINTER(Tuning)]
        l.dsrg_sprite_frame.argtypes = [P, C.POINTER(SpriteFrame)]
        l.dsrg_check_float_roots.argtypes = [P, C.c_uint32, C.c_uint32, C.POINTER(C.c_uint64)]
        _lib = l
    return _lib


def _torch_sync(*images):
    """Waits for torch's current stream: device tensors handed to the library may still be being
    written there, and the library works on its own stream.  (Every library call returns with
    its own work finished, so torch may read the results right after.)  Given the call's images,
    it waits only when one of them is a device tensor."""
    if images and all(a is None or isinstance(a, np.ndarray) for a in images):
        return
    import sys
    torch = sys.modules.get("torch")
    if torch is not None and torch.cuda.is_available() and torch.cuda.is_initialized():
        torch.cuda.current_stream().synchronize()


def _ptr(a) -> Optional[int]:
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    return int(a.data_ptr())  # torch tensor


def _row_bytes(a) -> int:
    """Row stride in bytes of a 2-D numpy array or torch tensor of 4-byte pixels."""
    return int(a.strides[0]) if isinstance(a, np.ndarray) else int(a.stride(0)) * 4


def camera_struct(scene) -> Camera:
    c = Camera()
    for i in range(12):
        c.location[i] = float(scene.camera_location[i])
    c.perspective = 1 if scene.perspective else 0
    c.slope = scene.slope
    c.nearClip = scene.near_clip
    c.farClip = scene.far_clip
    c.width = scene.width
    c.height = scene.height
    return c


# dsrg_projected_point: cs[3], is[2], flat[2] (int64 at offset 24)
PROJECTED_POINT = np.dtype({"names": ["cs", "is", "flat"], "formats": [("<f4", 3), ("<f4", 2), ("<i8", 2)],
                            "offsets": [0, 12, 24], "itemsize": 40})


def world_to_screen(camera: "Camera", world) -> np.ndarray:
    """dsrg_camera_world_to_screen of (..., 3) world points; returns PROJECTED_POINT records."""
    world = np.ascontiguousarray(world, np.float32)
    flat = world.reshape(-1, 3)
    out = np.zeros(len(flat), PROJECTED_POINT)
    l = lib()
    for i in range(len(flat)):
        status = l.dsrg_camera_world_to_screen(C.byref(camera), flat[i].ctypes.data, out[i:i + 1].ctypes.data)
        if status != DSRG_OK:
            raise DsrgError(status, "dsrg_camera_world_to_screen")
    return out.reshape(world.shape[:-1])


def image_struct(array, pack_order: int = 0) -> Optional[Image]:
    """A dsrg_image over a 2-D numpy array (host) or torch CUDA tensor (device) of 4-byte pixels."""
    if array is None:
        return None
    img = Image()
    if isinstance(array, np.ndarray):
        assert array.dtype.itemsize == 4 and array.ndim == 2 and array.strides[1] == 4
        img.data = array.ctypes.data
        img.height, img.width = array.shape
        img.strideBytes = array.strides[0]
        img.onDevice = 0
    else:
        assert array.element_size() == 4 and array.dim() == 2 and array.stride(1) == 1 and array.is_cuda
        img.data = array.data_ptr()
        img.height, img.width = array.shape
        img.strideBytes = array.stride(0) * 4
        img.onDevice = 1
    img.packOrder = pack_order
    return img


class Context:
    """A dsrg_context on one GPU."""

    def __init__(self, device: int = 0):
        self._l = lib()
        h = C.c_void_p()
        self._check(self._l.dsrg_context_create(device, C.byref(h)), None)
        self.handle = h
        self._children = weakref.WeakSet()

    def _adopt(self, child):
        self._children.add(child)

    def _check(self, status: int, handle=None):
        if status != DSRG_OK:
            msg = self._l.dsrg_context_last_error(handle if handle is not None else getattr(self, "handle", None))
            raise DsrgError(status, (msg or b"").decode())

    def close(self):
        """Destroys the context after every model, texture and renderer made from it."""
        if getattr(self, "handle", None):
            kids = list(self._children)
            for kind in (Diff, Batch, Renderer, Model, Texture):
                for child in kids:
                    if isinstance(child, kind):
                        child.destroy()
            self._l.dsrg_context_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def stream(self) -> int:
        return int(self._l.dsrg_context_stream(self.handle) or 0)

    def texture(self, pixels: np.ndarray, resolutions: int = 16) -> "Texture":
        return Texture(self, pixels, resolutions)

    def model(self, scene, diffuse: Optional["Texture"] = None, light: Optional["Texture"] = None) -> "Model":
        return Model(self, scene, diffuse, light)

    def set_counting(self, on: bool, coverage=None):
        self._check(self._l.dsrg_context_set_counting(self.handle, 1 if on else 0, _ptr(coverage)))

    def walked_fragments(self) -> int:
        """Fragments the tile kernels depth-tested on this context so far (early culling skips the rest)."""
        v = C.c_uint64()
        self._check(self._l.dsrg_context_walked_fragments(self.handle, C.byref(v)))
        return int(v.value)

    def stats(self) -> dict:
        s = Stats()
        self._check(self._l.dsrg_context_get_stats(self.handle, C.byref(s)))
        return {"fragments": int(s.fragments), "draw_records": int(s.drawRecords), "bin_entries": int(s.binEntries),
                "milliseconds": float(s.milliseconds), "raster_milliseconds": float(s.rasterMilliseconds),
                "kernel_launches": int(s.kernelLaunches)}

    def render(self, model: "Model", camera: Camera, color=None, depth=None, transform=None, pack_order: int = 0):
        """dsrg_model_render into the given host (numpy) or device (torch) images, in place."""
        t = np.ascontiguousarray(model.transform if transform is None else transform, np.float32)
        ci, di = image_struct(color, pack_order), image_struct(depth)
        _torch_sync(color, depth)
        self._check(self._l.dsrg_model_render(self.handle, model.handle, t.ctypes.data, C.byref(camera),
                                              C.byref(ci) if ci else None, C.byref(di) if di else None))

    def render_depth(self, model: "Model", camera: Camera, depth, transform=None):
        t = np.ascontiguousarray(model.transform if transform is None else transform, np.float32)
        di = image_struct(depth)
        _torch_sync()
        self._check(self._l.dsrg_model_render_depth(self.handle, model.handle, t.ctypes.data, C.byref(camera), C.byref(di)))

    def renderer(self) -> "Renderer":
        return Renderer(self)

    def batch(self) -> "Batch":
        return Batch(self)

    # ---- deferred light passes and draw_higher (torch CUDA tensors, or numpy arrays in host memory)

    def light_directed(self, view: "OrthoView", light, normal, direction, intensity: float, color, add: bool):
        d = np.asarray(direction, np.float32)
        c = np.asarray(color, np.int32)
        li, ni = image_struct(light), image_struct(normal)
        _torch_sync()
        self._check(self._l.dsrg_light_directed(self.handle, C.byref(view), C.byref(li), C.byref(ni), d.ctypes.data,
                                                C.c_float(intensity), c.ctypes.data, 1 if add else 0))

    @staticmethod
    def point_lights(lights):
        """A dsrg_point_light array from dicts with position, radius, intensity, color and optionally
        cube (cubeWidth*6 x cubeWidth floats)."""
        arr = (PointLight * max(1, len(lights)))()
        for i, l in enumerate(lights):
            for k in range(3):
                arr[i].position[k] = float(l["position"][k])
                arr[i].color[k] = int(l["color"][k])
            arr[i].radius = float(l["radius"])
            arr[i].intensity = float(l["intensity"])
            cube = l.get("cube")
            arr[i].shadowCube = _ptr(cube) if cube is not None else None
            arr[i].cubeWidth = int(cube.shape[1]) if cube is not None else 0
        return arr

    def light_points(self, view: "OrthoView", center, light, normal, height, lights, reference_threads: int = 0):
        """lights: dicts with position, radius, intensity, color and optionally cube (cubeWidth*6 x cubeWidth floats)."""
        arr = self.point_lights(lights)
        li, ni, hi = image_struct(light), image_struct(normal), image_struct(height)
        _torch_sync()
        self._check(self._l.dsrg_light_points(self.handle, C.byref(view), int(center[0]), int(center[1]), C.byref(li),
                                              C.byref(ni), C.byref(hi), arr, len(lights), reference_threads))

    def light_blend(self, target, diffuse, light, pack_order: int = 0):
        ti, di, li = image_struct(target, pack_order), image_struct(diffuse), image_struct(light)
        _torch_sync()
        self._check(self._l.dsrg_light_blend(self.handle, C.byref(ti), C.byref(di), C.byref(li)))

    def draw_higher(self, target_height, target_a, target_b, sprites, a_pack: int = 0, b_pack: int = 0):
        """sprites: a SpriteArray, or dicts with height, color_a, color_b (device tensors), left, top,
        offset, a_pack, b_pack."""
        array = sprites if isinstance(sprites, SpriteArray) else SpriteArray(sprites)
        hi, ai, bi = image_struct(target_height), image_struct(target_a, a_pack), image_struct(target_b, b_pack)
        _torch_sync()
        self._check(self._l.dsrg_draw_higher(self.handle, C.byref(hi), C.byref(ai), C.byref(bi), array.array, array.count))

    def check_float_roots(self, first_bits: int, count: int) -> int:
        """dsrg_check_float_roots: floats whose double-precision roots, rounded, differ from the
        correctly rounded single-precision ones."""
        out = C.c_uint64()
        self._check(self._l.dsrg_check_float_roots(self.handle, first_bits, count, C.byref(out)))
        return int(out.value)

    def sprite_frame(self, view: "OrthoView", center, images, clear, sprites, sun, shadows, lights, reference_threads: int = 0):
        """dsrg_sprite_frame: images = (height, diffuse, normal, light, output); clear = (height value,
        diffuse word, normal word); sprites a SpriteArray; sun = (direction, intensity, colour); shadows
        a depth-only Batch of cube faces or None; lights as for light_points."""
        structs = [image_struct(i) for i in images]
        lights_array = self.point_lights(lights)
        f = SpriteFrame()
        f.view = C.pointer(view)
        f.centerX, f.centerY = int(center[0]), int(center[1])
        f.height, f.diffuse, f.normal, f.light, f.output = [C.pointer(s) for s in structs]
        f.clearHeight, f.clearDiffuse, f.clearNormal = float(clear[0]), int(clear[1]), int(clear[2])
        f.sprites, f.spriteCount = sprites.array, sprites.count
        for k in range(3):
            f.sunDirection[k] = float(sun[0][k])
            f.sunColor[k] = int(sun[2][k])
        f.sunIntensity = float(sun[1])
        f.shadows = shadows.handle if shadows is not None else None
        f.lights, f.lightCount, f.referenceThreads = lights_array, len(lights), int(reference_threads)
        _torch_sync()
        self._check(self._l.dsrg_sprite_frame(self.handle, C.byref(f)))

    def dense_render(self, model: "DenseModel", view: "OrthoView", height, diffuse, normal, origin, model_to_world,
                     high_quality: bool = False):
        """renderDenseModel: the dense model drawn through the ortho view into device images (height
        F32, diffuse and normal RGBA) where it is higher; origin is the world origin in target pixels."""
        hi, di, ni = image_struct(height), image_struct(diffuse), image_struct(normal)
        t = np.ascontiguousarray(model_to_world, np.float32)
        _torch_sync()
        self._check(self._l.dsrg_dense_render(self.handle, model.handle, C.byref(view), C.byref(hi), C.byref(di), C.byref(ni),
                                              float(origin[0]), float(origin[1]), t.ctypes.data, 1 if high_quality else 0))

    def dense_render_many(self, instances, view: "OrthoView", height, diffuse, normal, high_quality: bool = False):
        """instances: (DenseModel, origin, model_to_world) in drawing order, drawn as that many
        dense_render calls would draw them, in one call."""
        arr = (DenseInstance * max(len(instances), 1))()
        for i, (model, origin, transform) in enumerate(instances):
            arr[i].model = model.handle
            arr[i].originX, arr[i].originY = float(origin[0]), float(origin[1])
            arr[i].modelToWorld[:] = [float(v) for v in np.asarray(transform, np.float32).reshape(12)]
        hi, di, ni = image_struct(height), image_struct(diffuse), image_struct(normal)
        _torch_sync()
        self._check(self._l.dsrg_dense_render_many(self.handle, arr, len(instances), C.byref(view), C.byref(hi), C.byref(di),
                                                   C.byref(ni), 1 if high_quality else 0))

    def tuning(self) -> dict:
        t = Tuning()
        self._check(self._l.dsrg_context_get_tuning(self.handle, C.byref(t)))
        return t.as_dict()

    def set_tuning(self, threads_per_tile: Optional[int] = None, ctas_per_sm: Optional[int] = None,
                   small_rows: Optional[int] = None, small_width: Optional[int] = None, graphs: Optional[bool] = None,
                   resolve: Optional[int] = None):
        t = Tuning()
        self._check(self._l.dsrg_context_get_tuning(self.handle, C.byref(t)))
        if threads_per_tile is not None:
            t.threadsPerTile = threads_per_tile
        if ctas_per_sm is not None:
            t.ctasPerSm = ctas_per_sm
        if small_rows is not None:
            t.smallRows = small_rows
        if small_width is not None:
            t.smallWidth = small_width
        if graphs is not None:
            t.graphs = 1 if graphs else 0
        if resolve is not None:
            t.resolve = resolve
        self._check(self._l.dsrg_context_set_tuning(self.handle, C.byref(t)))


class DenseInstance(C.Structure):
    _fields_ = [("model", C.c_void_p), ("originX", C.c_float), ("originY", C.c_float), ("modelToWorld", C.c_float * 12)]


class DenseModel:
    """DenseModel_create: a model's polygons as vertex-coloured triangles with smooth normals."""

    def __init__(self, ctx: Context, positions, polygons, colors):
        self.ctx = ctx
        pos = np.ascontiguousarray(positions, np.float32)
        poly = np.ascontiguousarray(polygons, np.int32)
        col = np.ascontiguousarray(colors, np.float32)
        h = C.c_void_p()
        ctx._check(ctx._l.dsrg_dense_model_create(ctx.handle, pos.ctypes.data, len(pos), poly.ctypes.data, col.ctypes.data, len(poly),
                                                  C.byref(h)))
        self.handle = h
        ctx._adopt(self)

    def destroy(self):
        if getattr(self, "handle", None) and self.ctx.handle:
            self.ctx._l.dsrg_dense_model_destroy(self.handle)
        self.handle = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass


class Texture:
    def __init__(self, ctx: Context, pixels: Optional[np.ndarray], resolutions: int = 16, handle=None):
        self.ctx = ctx
        if handle is None:
            pixels = np.ascontiguousarray(pixels, np.uint32)
            handle = C.c_void_p()
            ctx._check(ctx._l.dsrg_texture_create(ctx.handle, pixels.ctypes.data, pixels.shape[1], pixels.shape[0],
                                                  resolutions, C.byref(handle)))
        self.handle = handle
        ctx._adopt(self)

    @staticmethod
    def create_many(ctx: Context, images, resolutions, pack_orders=None) -> list:
        """dsrg_texture_create_many: images are (height, width) uint32 numpy arrays (host) or int32
        torch tensors (device); resolutions an int or one per image; pack_orders None (RGBA) or one
        per image."""
        n = len(images)
        res = [int(resolutions)] * n if np.isscalar(resolutions) else [int(r) for r in resolutions]
        structs = (Image * n)()
        keep = []
        for i, im in enumerate(images):
            if not hasattr(im, "data_ptr"):
                im = np.ascontiguousarray(im, np.uint32)
            keep.append(im)
            structs[i] = image_struct(im, 0 if pack_orders is None else int(pack_orders[i]))
        r = np.array(res, np.int32)
        out = (C.c_void_p * n)()
        _torch_sync()
        ctx._check(ctx._l.dsrg_texture_create_many(ctx.handle, n, structs, r.ctypes.data, out))
        return [Texture(ctx, None, handle=C.c_void_p(out[i])) for i in range(n)]

    def read(self):
        fields = np.zeros(9, np.uint32)
        count = C.c_int32()
        self.ctx._check(self.ctx._l.dsrg_texture_read(self.handle, None, 0, fields.ctypes.data, C.byref(count)))
        pixels = np.zeros(count.value, np.uint32)
        self.ctx._check(self.ctx._l.dsrg_texture_read(self.handle, pixels.ctypes.data, count.value, None, None))
        return fields, pixels

    def destroy(self):
        if getattr(self, "handle", None) and self.ctx.handle:
            self.ctx._l.dsrg_texture_destroy(self.handle)
        self.handle = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass


class Model:
    def __init__(self, ctx: Context, scene, diffuse: Optional[Texture] = None, light: Optional[Texture] = None):
        self.ctx = ctx
        self.scene = scene
        if diffuse is None and scene.diffuse is not None:
            diffuse = Texture(ctx, scene.diffuse, scene.diffuse_levels)
        if light is None and scene.light is not None:
            light = Texture(ctx, scene.light, scene.light_levels)
        self.diffuse, self.light = diffuse, light
        pos = np.ascontiguousarray(scene.positions, np.float32)
        poly = np.ascontiguousarray(scene.poly_indices, np.int32)
        tex = np.ascontiguousarray(scene.tex_coords, np.float32)
        col = np.ascontiguousarray(scene.colors, np.float32)
        h = C.c_void_p()
        ctx._check(ctx._l.dsrg_model_create(ctx.handle, pos.ctypes.data, pos.shape[0], poly.ctypes.data, tex.ctypes.data,
                                            col.ctypes.data, poly.shape[0], diffuse.handle if diffuse else None,
                                            light.handle if light else None, scene.filter, C.byref(h)))
        self.handle = h
        ctx._adopt(self)
        self.transform = np.ascontiguousarray(scene.model_to_world, np.float32)
        self.camera = camera_struct(scene)

    def destroy(self):
        if getattr(self, "handle", None) and self.ctx.handle:
            self.ctx._l.dsrg_model_destroy(self.handle)
        self.handle = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass


class Renderer:
    """dsrg_renderer: renderer_begin / renderer_giveTask / renderer_end."""

    def __init__(self, ctx: Context):
        self.ctx = ctx
        h = C.c_void_p()
        ctx._check(ctx._l.dsrg_renderer_create(ctx.handle, C.byref(h)))
        self.handle = h
        self._images = None
        ctx._adopt(self)

    def begin(self, color=None, depth=None, pack_order: int = 0):
        ci, di = image_struct(color, pack_order), image_struct(depth)
        self._images = (color, depth, ci, di)
        self.ctx._check(self.ctx._l.dsrg_renderer_begin(self.handle, C.byref(ci) if ci else None, C.byref(di) if di else None))

    def give_task(self, model: Model, camera: Optional[Camera] = None, transform=None):
        t = np.ascontiguousarray(model.transform if transform is None else transform, np.float32)
        cam = model.camera if camera is None else camera
        self.ctx._check(self.ctx._l.dsrg_renderer_give_task(self.handle, model.handle, t.ctypes.data, C.byref(cam)))

    def end(self, debug_wireframe: bool = False):
        _torch_sync(*(self._images[:2] if self._images else ()))
        if debug_wireframe:
            self.ctx._check(self.ctx._l.dsrg_renderer_end_debug(self.handle, 1))
        else:
            self.ctx._check(self.ctx._l.dsrg_renderer_end(self.handle))
        self._images = None

    @property
    def takes_triangles(self) -> bool:
        return bool(self.ctx._l.dsrg_renderer_takes_triangles(self.handle))

    def give_triangles(self, corners: np.ndarray, colors, tex_coords, diffuse: Optional["Texture"] = None,
                       light: Optional["Texture"] = None, filter: int = 0, camera: Optional[Camera] = None):
        """renderer_giveTask_triangle for n triangles: corners (n, 3) of PROJECTED_POINT, colors and
        tex_coords (n, 3, 4) float32."""
        corners = np.ascontiguousarray(corners, PROJECTED_POINT)
        colors = np.ascontiguousarray(colors, np.float32)
        tex = np.ascontiguousarray(tex_coords, np.float32)
        n = corners.shape[0]
        self.ctx._check(self.ctx._l.dsrg_renderer_give_triangles(
            self.handle, n, corners.ctypes.data, colors.ctypes.data, tex.ctypes.data, diffuse.handle if diffuse else None,
            light.handle if light else None, filter, C.byref(camera)))

    def images(self):
        c, dd = Image(), Image()
        self.ctx._check(self.ctx._l.dsrg_renderer_get_images(self.handle, C.byref(c), C.byref(dd)))
        return c, dd

    # the occlusion grid (renderer_occludeFromBox / FromExistingTriangles / FromTopRows, isBoxVisible)
    def occlude_from_box(self, minimum, maximum, transform, camera: Camera, debug_silhouette: bool = False):
        a, b = np.ascontiguousarray(minimum, np.float32), np.ascontiguousarray(maximum, np.float32)
        t = np.ascontiguousarray(transform, np.float32)
        self.ctx._check(self.ctx._l.dsrg_renderer_occlude_from_box(self.handle, a.ctypes.data, b.ctypes.data, t.ctypes.data,
                                                                   C.byref(camera), 1 if debug_silhouette else 0))

    def occlude_from_existing_triangles(self):
        self.ctx._check(self.ctx._l.dsrg_renderer_occlude_from_existing_triangles(self.handle))

    def occlude_from_top_rows(self, camera: Camera):
        _torch_sync()
        self.ctx._check(self.ctx._l.dsrg_renderer_occlude_from_top_rows(self.handle, C.byref(camera)))

    def is_box_visible(self, minimum, maximum, transform, camera: Camera) -> bool:
        a, b = np.ascontiguousarray(minimum, np.float32), np.ascontiguousarray(maximum, np.float32)
        t = np.ascontiguousarray(transform, np.float32)
        v = C.c_int32(0)
        self.ctx._check(self.ctx._l.dsrg_renderer_is_box_visible(self.handle, a.ctypes.data, b.ctypes.data, t.ctypes.data,
                                                                 C.byref(camera), C.byref(v)))
        return bool(v.value)

    @property
    def has_occluders(self) -> bool:
        return bool(self.ctx._l.dsrg_renderer_has_occluders(self.handle))

    def occlusion_grid(self) -> np.ndarray:
        gw, gh = C.c_int32(0), C.c_int32(0)
        self.ctx._check(self.ctx._l.dsrg_renderer_get_occlusion_grid(self.handle, None, 0, C.byref(gw), C.byref(gh)))
        out = np.zeros((gh.value, gw.value), np.float32)
        self.ctx._check(self.ctx._l.dsrg_renderer_get_occlusion_grid(self.handle, out.ctypes.data, out.size, C.byref(gw),
                                                                     C.byref(gh)))
        return out

    def destroy(self):
        if getattr(self, "handle", None) and self.ctx.handle:
            self.ctx._l.dsrg_renderer_destroy(self.handle)
        self.handle = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass


class SpriteArray:
    """A dsrg_sprite array built once from sprite dicts (see Context.draw_higher); it keeps the
    tensors it points at alive."""

    def __init__(self, sprites):
        self.count = len(sprites)
        self.array = (Sprite * max(1, self.count))()
        self._keep = []
        for i, sp in enumerate(sprites):
            h = sp["height"]
            a = self.array[i]
            a.height = _ptr(h)
            a.colorA = _ptr(sp["color_a"])
            a.colorB = _ptr(sp["color_b"])
            a.height_, a.width = int(h.shape[0]), int(h.shape[1])
            a.heightStrideBytes = _row_bytes(h)
            a.colorAStrideBytes = _row_bytes(sp["color_a"])
            a.colorBStrideBytes = _row_bytes(sp["color_b"])
            a.colorAPackOrder = int(sp.get("a_pack", 0))
            a.colorBPackOrder = int(sp.get("b_pack", 0))
            a.left, a.top = int(sp["left"]), int(sp["top"])
            a.offset = float(sp["offset"])
            a.onDevice = 0 if isinstance(h, np.ndarray) else 1
            self._keep.append((h, sp["color_a"], sp["color_b"]))


class Batch:
    """dsrg_batch: many frames, each its own renderer_begin ... renderer_end, drawn in one pass."""

    def __init__(self, ctx: Context):
        self.ctx = ctx
        h = C.c_void_p()
        ctx._check(ctx._l.dsrg_batch_create(ctx.handle, C.byref(h)))
        self.handle = h
        self._keep = []  # images and structs the library points at until the batch is cleared
        ctx._adopt(self)

    def add_frame(self, color=None, depth=None, pack_order: int = 0) -> int:
        ci, di = image_struct(color, pack_order), image_struct(depth)
        index = C.c_int32()
        self.ctx._check(self.ctx._l.dsrg_batch_add_frame(self.handle, C.byref(ci) if ci else None,
                                                         C.byref(di) if di else None, C.byref(index)))
        self._keep.append((color, depth))
        return index.value

    def give_task(self, frame: int, model: Model, camera: Optional[Camera] = None, transform=None):
        t = np.ascontiguousarray(model.transform if transform is None else transform, np.float32)
        cam = model.camera if camera is None else camera
        self.ctx._check(self.ctx._l.dsrg_batch_give_task(self.handle, frame, model.handle, t.ctypes.data, C.byref(cam)))
        self._keep.append(model)

    def render(self):
        _torch_sync()
        self.ctx._check(self.ctx._l.dsrg_batch_render(self.handle))

    def autotune(self, rounds: int = 2) -> dict:
        t = Tuning()
        _torch_sync()
        self.ctx._check(self.ctx._l.dsrg_batch_autotune(self.handle, rounds, C.byref(t)))
        return t.as_dict()

    def set_depth_only(self, on: bool):
        self.ctx._check(self.ctx._l.dsrg_batch_set_depth_only(self.handle, 1 if on else 0))

    def set_tuning(self, tuning: Optional[dict] = None):
        """dsrg_batch_set_tuning: this batch's own tile-kernel configuration (a dict as
        Context.tuning() returns; None: the context's)."""
        if tuning is None:
            self.ctx._check(self.ctx._l.dsrg_batch_set_tuning(self.handle, None))
            return
        t = Tuning(tuning["threads_per_tile"], tuning["ctas_per_sm"], tuning["small_rows"], tuning["small_width"],
                   int(tuning.get("graphs", 1)), tuning.get("resolve", 1))
        self.ctx._check(self.ctx._l.dsrg_batch_set_tuning(self.handle, C.byref(t)))

    def clear(self):
        self.ctx._check(self.ctx._l.dsrg_batch_clear(self.handle))
        self._keep = []

    def destroy(self):
        if getattr(self, "handle", None) and self.ctx.handle:
            self.ctx._l.dsrg_batch_destroy(self.handle)
        self.handle = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass


class Diff:
    """dsrg_diff: float-target rendering of one model with a visibility buffer, and its adjoint.

    Tensors are torch CUDA tensors (float32 / int32, contiguous): texture [th, tw, 4], vertex
    colours [points, 4], light [4] (dir xyz, intensity), images [views, h, w, 4], visibility
    [views, h, w, 3]."""

    def __init__(self, ctx: Context, model: Model, texture_width: int, texture_height: int, ambient: float):
        self.ctx = ctx
        self.model = model
        h = C.c_void_p()
        ctx._check(ctx._l.dsrg_diff_create(ctx.handle, model.handle, texture_width, texture_height, C.c_float(ambient),
                                           C.byref(h)))
        self.handle = h
        ctx._adopt(self)

    @staticmethod
    def _cameras(cameras):
        arr = (Camera * len(cameras))()
        for i, c in enumerate(cameras):
            arr[i] = c
        return arr

    def forward(self, cameras, transform, texture, vertex_colors, light, images, visibility):
        cams = self._cameras(cameras)
        t = np.ascontiguousarray(transform, np.float32)
        _torch_sync()
        self.ctx._check(self.ctx._l.dsrg_diff_forward(self.handle, len(cameras), cams, t.ctypes.data, _ptr(texture),
                                                      _ptr(vertex_colors), _ptr(light), _ptr(images), _ptr(visibility)))

    def l2_loss(self, images, targets, grad_images, loss):
        _torch_sync()
        self.ctx._check(self.ctx._l.dsrg_diff_l2_loss(self.handle, images.numel(), _ptr(images), _ptr(targets),
                                                      _ptr(grad_images), _ptr(loss)))

    def adjoint(self, views, width, height, transform, texture, vertex_colors, light, visibility, grad_images,
                grad_texture, grad_vertex_colors, grad_light, deterministic: bool = False):
        t = np.ascontiguousarray(transform, np.float32)
        _torch_sync()
        self.ctx._check(self.ctx._l.dsrg_diff_adjoint(self.handle, views, width, height, t.ctypes.data, _ptr(texture),
                                                      _ptr(vertex_colors), _ptr(light), _ptr(visibility), _ptr(grad_images),
                                                      _ptr(grad_texture), _ptr(grad_vertex_colors), _ptr(grad_light),
                                                      1 if deterministic else 0))

    def destroy(self):
        if getattr(self, "handle", None) and self.ctx.handle:
            self.ctx._l.dsrg_diff_destroy(self.handle)
        self.handle = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass


def ortho_view(camera_tilt: float, pixels_per_tile: int, index: int) -> OrthoView:
    """OrthoSystem(cameraTilt, pixelsPerTile).view[index] (host computation, no GPU)."""
    v = OrthoView()
    status = lib().dsrg_ortho_view_create(camera_tilt, pixels_per_tile, index, C.byref(v))
    if status != DSRG_OK:
        raise DsrgError(status, "dsrg_ortho_view_create")
    return v


def shadow_side_location(normal_to_world, side: int) -> np.ndarray:
    n = np.ascontiguousarray(normal_to_world, np.float32)
    out = np.zeros(12, np.float32)
    status = lib().dsrg_shadow_side_location(n.ctypes.data, side, out.ctypes.data)
    if status != DSRG_OK:
        raise DsrgError(status, "dsrg_shadow_side_location")
    return out


def render_scene(ctx: Context, scene, color: Optional[np.ndarray] = None, depth: Optional[np.ndarray] = None, *,
                 use_color: bool = True, use_depth: bool = True, pack_order: int = 0, model: Optional[Model] = None):
    """Renders a scene into fresh (or given) host images through dsrg_model_render; returns (color, depth)."""
    m = model or Model(ctx, scene)
    h, w = scene.height, scene.width
    c = (np.zeros((h, w), np.uint32) if color is None else np.array(color, np.uint32)) if use_color else None
    d = (np.zeros((h, w), np.float32) if depth is None else np.array(depth, np.float32)) if use_depth else None
    ctx.render(m, m.camera, c, d, pack_order=pack_order)
    return c, d
