"""pixie's raster hot path on a GB300, behind pixie's own API shape.

``Image`` mirrors pixie's Image (src/pixie/common.nim:34-37) with its pixels
resident in GPU memory; its methods are the reference's fillPath,
strokePath, draw, blur, shadow and fill (src/pixie/paths.nim:2093-2175,
src/pixie/images.nim:55-776), executed by the CUDA library libpxg.so through
the C ABI declared in include/pxg.h.  There is no CPU fallback: constructing
an Image fails loudly if the library or the GPU is unavailable.
"""
from __future__ import annotations

import ctypes as C
import enum
import os

import numpy as np

from .paths import Path, PixieError, as_commands, parse_path  # noqa: F401

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libpxg.so")


class BlendMode(enum.IntEnum):  # common.nim:6-29
    NormalBlend = 0
    DarkenBlend = 1
    MultiplyBlend = 2
    ColorBurnBlend = 3
    LightenBlend = 4
    ScreenBlend = 5
    ColorDodgeBlend = 6
    OverlayBlend = 7
    SoftLightBlend = 8
    HardLightBlend = 9
    DifferenceBlend = 10
    ExclusionBlend = 11
    HueBlend = 12
    SaturationBlend = 13
    ColorBlend = 14
    LuminosityBlend = 15
    MaskBlend = 16
    OverwriteBlend = 17
    SubtractMaskBlend = 18
    ExcludeMaskBlend = 19


class WindingRule(enum.IntEnum):  # paths.nim:5-8
    NonZero = 0
    EvenOdd = 1


class LineCap(enum.IntEnum):  # paths.nim:10-12
    ButtCap = 0
    RoundCap = 1
    SquareCap = 2


class LineJoin(enum.IntEnum):  # paths.nim:14-16
    MiterJoin = 0
    RoundJoin = 1
    BevelJoin = 2


DEFAULT_MITER_LIMIT = 4.0  # paths.nim:46

_lib = None


def lib():
    """The loaded libpxg.so (raises if it is missing: no CPU fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise PixieError(f"libpxg.so is not built ({LIB_PATH}); run python -m pixie_gb300.build")
        L = C.CDLL(LIB_PATH)
        P, I64, F, I = C.c_void_p, C.c_int64, C.c_float, C.c_int
        L.pxg_take_error.restype = C.c_char_p
        L.pxg_init.argtypes = [I]
        L.pxg_set_stream.argtypes = [P]
        L.pxg_new_image.restype = P
        L.pxg_new_image.argtypes = [I64, I64]
        L.pxg_image_wrap.restype = P
        L.pxg_image_wrap.argtypes = [P, I64, I64]
        L.pxg_image_free.argtypes = [P]
        L.pxg_image_free.restype = None
        L.pxg_image_width.argtypes = [P]
        L.pxg_image_width.restype = I64
        L.pxg_image_height.argtypes = [P]
        L.pxg_image_height.restype = I64
        L.pxg_image_device_ptr.argtypes = [P]
        L.pxg_image_device_ptr.restype = P
        L.pxg_image_upload.argtypes = [P, P, I64]
        L.pxg_image_download.argtypes = [P, P, I64]
        L.pxg_image_fill.argtypes = [P, P]
        L.pxg_image_fill_path.argtypes = [P, P, I64, P, F, I, P, I]
        L.pxg_image_stroke_path.argtypes = [P, P, I64, P, F, I, P, F, I, I, F, P, I64]
        L.pxg_image_draw.argtypes = [P, P, I64, I64, I]
        L.pxg_image_draw_transform.argtypes = [P, P, P, I]
        L.pxg_image_draw_tiled.argtypes = [P, P, P, I]
        L.pxg_image_fill_path_paint.argtypes = [P, P, I64, P, P, I]
        L.pxg_image_stroke_path_paint.argtypes = [P, P, I64, P, P, F, I, I, F, P, I64]
        L.pxg_image_fill_paint.argtypes = [P, P]
        L.pxg_image_minify_by2.argtypes = [P, I]
        L.pxg_image_minify_by2.restype = P
        L.pxg_image_magnify_by2.argtypes = [P, I]
        L.pxg_image_magnify_by2.restype = P
        L.pxg_image_blur.argtypes = [P, F, P]
        L.pxg_image_spread.argtypes = [P, F]
        L.pxg_image_shadow.argtypes = [P, F, F, F, F, P]
        L.pxg_image_shadow.restype = P
        L.pxg_image_shadow_into.argtypes = [P, P, F, F, F, F, P]
        L.pxg_set_blocking.argtypes = [I]
        L.pxg_launch_count.restype = I64
        L.pxg_blend_pixels.argtypes = [I, P, P, P, I64]
        L.pxg_fill_paths_batch.argtypes = [P, I64, P, P, P, P, P, P, P, P]
        L.pxg_last_gpu_ms.restype = F
        L.pxg_scene_new.restype = P
        L.pxg_scene_free.argtypes = [P]
        L.pxg_scene_free.restype = None
        L.pxg_scene_clear.argtypes = [P]
        L.pxg_scene_len.argtypes = [P]
        L.pxg_scene_len.restype = I64
        L.pxg_scene_fill_path.argtypes = [P, P, I64, P, F, I, P, I]
        L.pxg_scene_stroke_path.argtypes = [P, P, I64, P, F, I, P, F, I, I, F, P, I64]
        L.pxg_scene_record_batch.argtypes = [P, I64, P, P, P, P, P, P, P, P, P, P, P, P, P, I]
        L.pxg_masks_add_paths.argtypes = [P, I64, P, P, P, P, P, P, I]
        L.pxg_image_draw_scene.argtypes = [P, P]
        L.pxg_scene_config.argtypes = [I, I64]
        L.pxg_last_fill_stats.argtypes = [P]
        L.pxg_masks_new.restype = P
        L.pxg_masks_free.argtypes = [P]
        L.pxg_masks_free.restype = None
        L.pxg_masks_len.argtypes = [P]
        L.pxg_masks_len.restype = I64
        L.pxg_masks_add_path.argtypes = [P, P, I64, I64, I64, P, I]
        L.pxg_masks_render.argtypes = [P]
        L.pxg_masks_render_config.argtypes = [P, I, I]
        L.pxg_masks_download.argtypes = [P, I64, P, I64]
        L.pxg_masks_device_ptr.argtypes = [P, I64]
        L.pxg_masks_device_ptr.restype = P
        L.pxg_image_draw_masks.argtypes = [P, P, P, I]
        L.pxg_server_new.restype = P
        L.pxg_server_new.argtypes = [I64, I64, I64]
        L.pxg_server_free.argtypes = [P]
        L.pxg_server_free.restype = None
        L.pxg_server_submit.argtypes = [P, P, I64, I64, F]
        L.pxg_server_submit.restype = I64
        L.pxg_server_step.argtypes = [P]
        L.pxg_server_pending.argtypes = [P]
        L.pxg_server_pending.restype = I64
        L.pxg_server_poll.argtypes = [P, P, I64]
        L.pxg_server_poll.restype = I64
        L.pxg_server_take.argtypes = [P, I64, P, I64, P]
        L.pxg_server_stats.argtypes = [P, P]
        L.pxg_autotune.argtypes = [I]
        L.pxg_blur_config.argtypes = [I]
        L.pxg_stroke_config.argtypes = [I]
        L.pxg_image_apply_opacity.argtypes = [P, F]
        L.pxg_stroke_fixups.restype = I64
        L.pxg_ring_trace.argtypes = [I, P, I64]
        L.pxg_autotune_report.argtypes = [P, I64]
        L.pxg_autotune_report.restype = I64
        _lib = L
    return _lib


def _check(rc: int):
    if rc != 0:
        raise PixieError(lib().pxg_take_error().decode())


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def _color(c) -> np.ndarray:
    return np.ascontiguousarray(c, dtype=np.float32).reshape(4)


def _mat(m):
    if m is None:
        return None
    return np.ascontiguousarray(m, dtype=np.float32).reshape(9)


def rgba(r, g, b, a=255):
    """ColorRGBA as a paint colour: chroma's Color is c / 255 in float32."""
    return [np.float32(v) / np.float32(255) for v in (r, g, b, a)]


def translate(x, y):
    return np.array([1, 0, 0, 0, 1, 0, x, y, 1], dtype=np.float32)


def scale(x, y):
    return np.array([x, 0, 0, 0, y, 0, 0, 0, 1], dtype=np.float32)


class PaintKind(enum.IntEnum):  # paints.nim:4-10
    SolidPaint = 0
    ImagePaint = 1
    TiledImagePaint = 2
    LinearGradientPaint = 3
    RadialGradientPaint = 4
    AngularGradientPaint = 5


class _CPaint(C.Structure):  # pxg_paint (include/pxg.h)
    _fields_ = [("kind", C.c_int32), ("blend_mode", C.c_int32), ("opacity", C.c_float),
                ("color", C.c_float * 4), ("image", C.c_void_p), ("image_mat", C.c_float * 9),
                ("n_handles", C.c_int32), ("handles", C.c_void_p), ("n_stops", C.c_int32),
                ("stops", C.c_void_p)]


class Paint:
    """A paint (paints.nim:12-26): a solid colour, an image (imageMat places it,
    tiled or not) or a linear / radial / angular gradient (handle positions in
    image space, colour stops (color, position)); opacity and blend mode."""

    def __init__(self, color=(0, 0, 0, 1), opacity=1.0, blend_mode=BlendMode.NormalBlend,
                 kind=PaintKind.SolidPaint, image=None, image_mat=None, handles=(), stops=()):
        self.kind = kind
        self.color = color
        self.opacity = opacity
        self.blend_mode = blend_mode
        self.image = image
        self.image_mat = image_mat
        self.handles = list(handles)
        self.stops = list(stops)

    def _c(self):
        """(the pxg_paint struct, arrays it points into, kept alive by the caller)"""
        cp = _CPaint()
        cp.kind, cp.blend_mode, cp.opacity = int(self.kind), int(self.blend_mode), float(self.opacity)
        cp.color[:] = [float(v) for v in _color(self.color)]
        cp.image = self.image._h if self.image is not None else None
        cp.image_mat[:] = [float(v) for v in (_mat(self.image_mat) if self.image_mat is not None
                                              else np.array([1, 0, 0, 0, 1, 0, 0, 0, 1], np.float32))]
        h = np.ascontiguousarray(np.asarray(self.handles, np.float32).reshape(-1))
        st = np.ascontiguousarray(np.asarray([list(c) + [pos] for c, pos in self.stops], np.float32).reshape(-1))
        cp.n_handles, cp.handles = len(self.handles), (h.ctypes.data if h.size else None)
        cp.n_stops, cp.stops = len(self.stops), (st.ctypes.data if st.size else None)
        return cp, (h, st)


def _paint(p):
    if isinstance(p, Paint):
        return _color(p.color), float(p.opacity), int(p.blend_mode)
    return _color(p), 1.0, int(BlendMode.NormalBlend)


class Image:
    """A premultiplied RGBX image resident in GPU memory."""

    def __init__(self, width: int, height: int, _handle=None):
        if _handle is None:
            _handle = lib().pxg_new_image(int(width), int(height))
            if not _handle:
                raise PixieError(lib().pxg_take_error().decode())
        self._h = _handle
        self.width = int(lib().pxg_image_width(self._h))
        self.height = int(lib().pxg_image_height(self._h))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and _lib is not None:
            _lib.pxg_image_free(h)
            self._h = None

    @classmethod
    def from_numpy(cls, arr: np.ndarray) -> "Image":
        img = cls(arr.shape[1], arr.shape[0])
        img.upload(arr)
        return img

    @classmethod
    def wrap(cls, device_ptr: int, width: int, height: int) -> "Image":
        h = lib().pxg_image_wrap(C.c_void_p(device_ptr), int(width), int(height))
        if not h:
            raise PixieError(lib().pxg_take_error().decode())
        return cls(width, height, _handle=h)

    @property
    def device_ptr(self) -> int:
        return int(lib().pxg_image_device_ptr(self._h))

    def to_numpy(self) -> np.ndarray:
        out = np.empty((self.height, self.width, 4), dtype=np.uint8)
        _check(lib().pxg_image_download(self._h, _ptr(out), out.nbytes))
        if not _blocking:  # an asynchronous download: wait for it before handing the array out
            _check(lib().pxg_synchronize())
        return out

    def upload(self, arr: np.ndarray):
        arr = np.ascontiguousarray(arr, dtype=np.uint8)
        _check(lib().pxg_image_upload(self._h, _ptr(arr), arr.nbytes))
        if not _blocking:  # an asynchronous upload reads the host bytes until pxg_synchronize
            _pending_uploads.append(arr)

    # -- pixie's Image procs -------------------------------------------------
    def fill(self, color):
        """fill with a colour (images.nim:55-57) or a Paint (pixie.nim:120-131)"""
        if isinstance(color, Paint):
            cp, keep = color._c()
            _check(lib().pxg_image_fill_paint(self._h, C.byref(cp)))
            return
        _check(lib().pxg_image_fill(self._h, _ptr(_color(color))))

    def fill_path(self, path, paint, transform=None, winding_rule=WindingRule.NonZero):
        cmds = as_commands(path)
        m = _mat(transform)
        if isinstance(paint, Paint) and paint.kind != PaintKind.SolidPaint:
            cp, keep = paint._c()
            _check(lib().pxg_image_fill_path_paint(self._h, _ptr(cmds), cmds.size, C.byref(cp),
                                                   None if m is None else _ptr(m), int(winding_rule)))
            return
        col, op, blend = _paint(paint)
        _check(lib().pxg_image_fill_path(self._h, _ptr(cmds), cmds.size, _ptr(col), op, blend,
                                         None if m is None else _ptr(m), int(winding_rule)))

    def stroke_path(self, path, paint, transform=None, stroke_width=1.0,
                    line_cap=LineCap.ButtCap, line_join=LineJoin.MiterJoin,
                    miter_limit=DEFAULT_MITER_LIMIT, dashes=()):
        cmds = as_commands(path)
        m = _mat(transform)
        d = np.ascontiguousarray(list(dashes) if len(dashes) else [0.0], dtype=np.float32)
        if isinstance(paint, Paint) and paint.kind != PaintKind.SolidPaint:
            cp, keep = paint._c()
            _check(lib().pxg_image_stroke_path_paint(self._h, _ptr(cmds), cmds.size, C.byref(cp),
                                                     None if m is None else _ptr(m), float(stroke_width),
                                                     int(line_cap), int(line_join), float(miter_limit),
                                                     _ptr(d), len(dashes)))
            return
        col, op, blend = _paint(paint)
        _check(lib().pxg_image_stroke_path(self._h, _ptr(cmds), cmds.size, _ptr(col), op, blend,
                                           None if m is None else _ptr(m), float(stroke_width),
                                           int(line_cap), int(line_join), float(miter_limit),
                                           _ptr(d), len(dashes)))

    def draw(self, b: "Image", translate_xy=(0, 0), blend_mode=BlendMode.NormalBlend):
        """draw(a, b, translate(x, y), mode): whole-pixel offsets take blendRect,
        fractional ones drawSmooth (images.nim:636-678)."""
        tx, ty = translate_xy
        if tx != int(tx) or ty != int(ty):
            self.draw_transform(b, [1, 0, 0, 0, 1, 0, tx, ty, 1], blend_mode)
            return
        _check(lib().pxg_image_draw(self._h, b._h, int(tx), int(ty), int(blend_mode)))

    def draw_transform(self, b: "Image", transform, blend_mode=BlendMode.NormalBlend):
        """draw(a, b, transform: Mat3, mode); transform is 9 floats, column-major
        like vmath's Mat3 (translation in [6], [7])."""
        m = np.ascontiguousarray(np.asarray(transform, dtype=np.float32).reshape(9))
        _check(lib().pxg_image_draw_transform(self._h, b._h, _ptr(m), int(blend_mode)))

    def draw_tiled(self, b: "Image", transform, blend_mode=BlendMode.NormalBlend):
        """drawTiled(a, b, transform, mode) (images.nim:680-683)"""
        m = np.ascontiguousarray(np.asarray(transform, dtype=np.float32).reshape(9))
        _check(lib().pxg_image_draw_tiled(self._h, b._h, _ptr(m), int(blend_mode)))

    def minify_by2(self, power: int = 1) -> "Image":
        h = lib().pxg_image_minify_by2(self._h, int(power))
        if not h:
            raise PixieError(lib().pxg_take_error().decode())
        return Image(0, 0, _handle=h)

    def magnify_by2(self, power: int = 1) -> "Image":
        h = lib().pxg_image_magnify_by2(self._h, int(power))
        if not h:
            raise PixieError(lib().pxg_take_error().decode())
        return Image(0, 0, _handle=h)

    def blur(self, radius: float, out_of_bounds=(0, 0, 0, 0)):
        _check(lib().pxg_image_blur(self._h, float(radius), _ptr(_color(out_of_bounds))))

    def apply_opacity(self, opacity: float):
        """applyOpacity (images.nim:261-277)"""
        _check(lib().pxg_image_apply_opacity(self._h, float(opacity)))

    def spread(self, spread: float):
        _check(lib().pxg_image_spread(self._h, float(spread)))

    def shadow(self, offset, spread: float, blur: float, color) -> "Image":
        h = lib().pxg_image_shadow(self._h, float(offset[0]), float(offset[1]), float(spread),
                                   float(blur), _ptr(_color(color)))
        if not h:
            raise PixieError(lib().pxg_take_error().decode())
        return Image(0, 0, _handle=h)

    def shadow_into(self, out: "Image", offset, spread: float, blur: float, color):
        _check(lib().pxg_image_shadow_into(self._h, out._h, float(offset[0]), float(offset[1]),
                                           float(spread), float(blur), _ptr(_color(color))))


    def draw_masks(self, masks: "Masks", positions, blend_mode=BlendMode.NormalBlend):
        draw_masks(self, masks, positions, blend_mode)

    def draw_scene(self, scene: "Scene"):
        """Paints the scene's recorded paths in order (one setup and one row
        launch for the whole sequence)."""
        _check(lib().pxg_image_draw_scene(self._h, scene._h))


class Scene:
    """A recorded sequence of fill_path/stroke_path calls, painted in order
    onto an image by Image.draw_scene.  Each call takes the arguments of the
    Image method of the same name."""

    def __init__(self):
        self._h = lib().pxg_scene_new()
        if not self._h:
            raise PixieError(lib().pxg_take_error().decode())

    def __del__(self):
        h, self._h = getattr(self, "_h", None), None
        if h and _lib is not None:
            _lib.pxg_scene_free(h)

    def record_batch(self, paths, threads: int = 0) -> np.ndarray:
        """Records many fill_path / stroke_path calls at once, their geometry
        built on host threads and appended in order.  Each path is a dict:
        kind ("fill" or "stroke"), cmds, color, opacity (1), blend (0),
        transform (None), winding (fills), width / cap / join / miter (strokes).
        Returns the per-path status (1 where the path failed and was skipped)."""
        n = len(paths)
        cm = [as_commands(p["cmds"]) for p in paths]
        offs = np.zeros(n + 1, np.int64)
        offs[1:] = np.cumsum([c.size for c in cm])
        cmds = np.ascontiguousarray(np.concatenate(cm) if n else np.zeros(1, np.float32), dtype=np.float32)
        kinds = np.array([0 if p["kind"] == "fill" else 1 for p in paths], np.int32)
        colors = np.ascontiguousarray(np.array([_color(p["color"]) for p in paths], np.float32).reshape(-1))
        ops = np.array([p.get("opacity", 1.0) for p in paths], np.float32)
        blends = np.array([int(p.get("blend", 0)) for p in paths], np.int32)
        has_t = any(p.get("transform") is not None for p in paths)
        mats = (np.ascontiguousarray(np.array([_mat(p.get("transform")) if p.get("transform") is not None
                                               else np.array([1, 0, 0, 0, 1, 0, 0, 0, 1], np.float32)
                                               for p in paths], np.float32).reshape(-1)) if has_t else None)
        wind = np.array([int(p.get("winding", 0)) for p in paths], np.int32)
        widths = np.array([p.get("width", 1.0) for p in paths], np.float32)
        caps = np.array([int(p.get("cap", 0)) for p in paths], np.int32)
        joins = np.array([int(p.get("join", 0)) for p in paths], np.int32)
        miters = np.array([p.get("miter", DEFAULT_MITER_LIMIT) for p in paths], np.float32)
        status = np.zeros(max(n, 1), np.int32)
        _check(lib().pxg_scene_record_batch(self._h, n, _ptr(kinds), _ptr(cmds), _ptr(offs), _ptr(colors),
                                            _ptr(ops), _ptr(blends), None if mats is None else _ptr(mats),
                                            _ptr(wind), _ptr(widths), _ptr(caps), _ptr(joins), _ptr(miters),
                                            _ptr(status), int(threads)))
        return status[:n]

    def __len__(self):
        return int(lib().pxg_scene_len(self._h))

    def clear(self):
        _check(lib().pxg_scene_clear(self._h))

    def fill_path(self, path, paint, transform=None, winding_rule=WindingRule.NonZero):
        cmds = as_commands(path)
        col, op, blend = _paint(paint)
        m = _mat(transform)
        _check(lib().pxg_scene_fill_path(self._h, _ptr(cmds), cmds.size, _ptr(col), op, blend,
                                         None if m is None else _ptr(m), int(winding_rule)))

    def stroke_path(self, path, paint, transform=None, stroke_width=1.0,
                    line_cap=LineCap.ButtCap, line_join=LineJoin.MiterJoin,
                    miter_limit=DEFAULT_MITER_LIMIT, dashes=()):
        cmds = as_commands(path)
        col, op, blend = _paint(paint)
        m = _mat(transform)
        d = np.ascontiguousarray(list(dashes) if len(dashes) else [0.0], dtype=np.float32)
        _check(lib().pxg_scene_stroke_path(self._h, _ptr(cmds), cmds.size, _ptr(col), op, blend,
                                           None if m is None else _ptr(m), float(stroke_width),
                                           int(line_cap), int(line_join), float(miter_limit),
                                           _ptr(d), len(dashes)))


class Masks:
    """A batch of 8-bit masks: add_path(path, width, height) fills the path
    with color(1, 1, 1, 1) on a transparent width x height image and keeps its
    alpha; render() renders the whole batch on the GPU (one graph launch);
    Image.draw_masks composites them in order."""

    def __init__(self):
        self._h = lib().pxg_masks_new()
        if not self._h:
            raise PixieError(lib().pxg_take_error().decode())
        self._sizes = []

    def __del__(self):
        h, self._h = getattr(self, "_h", None), None
        if h and _lib is not None:
            _lib.pxg_masks_free(h)

    def __len__(self):
        return int(lib().pxg_masks_len(self._h))

    def add_path(self, path, width: int, height: int, transform=None,
                 winding_rule=WindingRule.NonZero):
        cmds = as_commands(path)
        m = _mat(transform)
        _check(lib().pxg_masks_add_path(self._h, _ptr(cmds), cmds.size, int(width), int(height),
                                        None if m is None else _ptr(m), int(winding_rule)))
        self._sizes.append((int(width), int(height)))

    def add_paths(self, paths, threads: int = 0):
        """add_path for many glyphs at once: (path, width, height, winding_rule)
        tuples, geometry built on host threads, masks appended in order (all
        or nothing)."""
        n = len(paths)
        cm = [as_commands(p[0]) for p in paths]
        offs = np.zeros(n + 1, np.int64)
        offs[1:] = np.cumsum([c.size for c in cm])
        cmds = np.ascontiguousarray(np.concatenate(cm) if n else np.zeros(1, np.float32), dtype=np.float32)
        ws = np.array([int(p[1]) for p in paths], np.int64)
        hs = np.array([int(p[2]) for p in paths], np.int64)
        wind = np.array([int(p[3]) if len(p) > 3 else 0 for p in paths], np.int32)
        _check(lib().pxg_masks_add_paths(self._h, n, _ptr(cmds), _ptr(offs), _ptr(ws), _ptr(hs), None,
                                         _ptr(wind), int(threads)))
        self._sizes.extend(zip(ws.tolist(), hs.tolist()))

    def render(self):
        _check(lib().pxg_masks_render(self._h))

    def render_config(self, variant: int, rows_per_item: int):
        """Renders with a fixed row-kernel configuration (tests, tuning)."""
        _check(lib().pxg_masks_render_config(self._h, int(variant), int(rows_per_item)))

    def mask(self, i: int) -> np.ndarray:
        w, h = self._sizes[i]
        out = np.empty((h, w), np.uint8)
        _check(lib().pxg_masks_download(self._h, int(i), _ptr(out), out.nbytes))
        return out


def draw_masks(page: "Image", masks: Masks, positions, blend_mode=BlendMode.NormalBlend):
    """draw(page, mask_i, translate(x_i, y_i), blend_mode) for every mask in order."""
    xy = np.ascontiguousarray(positions, np.int64).reshape(-1, 2)
    if len(xy) != len(masks):
        raise PixieError("one position per mask is required")
    _check(lib().pxg_image_draw_masks(page._h, masks._h, _ptr(xy), int(blend_mode)))


class Server:
    """Continuous-batching render server (see pxg_server_* in include/pxg.h).
    submit(scene, width, height, blur) -> job id; step() advances admitted
    jobs; poll() -> finished ids; take(id) -> (canvas RGBX array or None,
    (submit, admit, done) times)."""

    def __init__(self, budget_bytes=40 << 30, paths_per_job=512, paths_per_step=16384):
        self._h = lib().pxg_server_new(int(budget_bytes), int(paths_per_job), int(paths_per_step))
        if not self._h:
            raise PixieError(lib().pxg_take_error().decode())
        self._scenes = {}
        self._sizes = {}

    def __del__(self):
        h, self._h = getattr(self, "_h", None), None
        if h and _lib is not None:
            _lib.pxg_server_free(h)

    def submit(self, scene: "Scene", width: int, height: int, blur: float = 0.0) -> int:
        jid = int(lib().pxg_server_submit(self._h, scene._h, int(width), int(height), float(blur)))
        if jid == 0:
            raise PixieError(lib().pxg_take_error().decode())
        self._scenes[jid] = scene  # kept alive until taken
        self._sizes[jid] = (int(width), int(height))
        return jid

    def step(self):
        _check(lib().pxg_server_step(self._h))

    def pending(self) -> int:
        return int(lib().pxg_server_pending(self._h))

    def poll(self, cap: int = 4096):
        ids = np.zeros(cap, np.int64)
        n = int(lib().pxg_server_poll(self._h, _ptr(ids), cap))
        return [int(v) for v in ids[:n]]

    def take(self, jid: int, download: bool = True):
        w, h = self._sizes[jid]
        out = np.empty((h, w, 4), np.uint8) if download else None
        times = np.zeros(3, np.float64)
        try:
            _check(lib().pxg_server_take(self._h, int(jid), None if out is None else _ptr(out),
                                         0 if out is None else out.nbytes, _ptr(times)))
        finally:
            self._scenes.pop(jid, None)
            self._sizes.pop(jid, None)
        return out, tuple(float(t) for t in times)

    def stats(self) -> dict:
        v = np.zeros(6, np.int64)
        _check(lib().pxg_server_stats(self._h, _ptr(v)))
        return dict(zip(["steps", "bytes_used", "peak_bytes", "peak_admitted", "queued", "admitted"],
                        [int(x) for x in v]))


def scene_config(slice_width: int = 256, coverage_bytes: int = -1):
    """Scene drawing configuration (see pxg_scene_config)."""
    _check(lib().pxg_scene_config(int(slice_width), int(coverage_bytes)))


def stroke_config(gpu_outline: bool):
    """True (default): strokes without dashes are outlined on the GPU; False:
    every outline is built on the host (see pxg_stroke_config)."""
    _check(lib().pxg_stroke_config(1 if gpu_outline else 0))


def stroke_fixups() -> int:
    """Joins of GPU outlines rebuilt on the host since the library loaded."""
    return int(lib().pxg_stroke_fixups())


def blur_config(mode):
    """3 (default): tensor-core blur with TMA-fed input rings (radii 1..128,
    rows a multiple of 16 bytes); 1: the pipelined tensor-core kernel that
    loads through registers (radii 8..128); 2: the single-stage tensor-core
    kernel (radii 8..128); 0: CUDA cores.  Radii or images a mode does not
    take run on the next family (3 -> 1 -> 0)."""
    _check(lib().pxg_blur_config(int(mode)))


def last_blur_kernel() -> int:
    """Kernel family the last blur ran on (3, 2, 1, 0; -1 before any)."""
    return int(lib().pxg_last_blur_kernel())


def ring_trace(enable: bool, fetch: bool = False):
    """The ring blur passes' converter trace (a profiling aid; see
    pxg_ring_trace in include/pxg.h): switch it on or off; with fetch, the
    last traced pass's clock64 stamps as an int64 array [group][chunk][event]."""
    out = np.zeros((2, 256, 3), np.int64) if fetch else None
    _check(lib().pxg_ring_trace(1 if enable else 0, None if out is None else _ptr(out),
                                0 if out is None else out.size))
    return out


def autotune(enable: bool):
    _check(lib().pxg_autotune(1 if enable else 0))


def autotune_report() -> str:
    n = int(lib().pxg_autotune_report(None, 0))
    buf = C.create_string_buffer(n + 1)
    lib().pxg_autotune_report(buf, n + 1)
    return buf.value.decode()


def blend_pixels(mode: int, backdrop_dev: int, source_dev: int, out_dev: int, n: int):
    """blender(mode) over n device pixels (for testing the blend modes)."""
    _check(lib().pxg_blend_pixels(int(mode), C.c_void_p(backdrop_dev), C.c_void_p(source_dev),
                                  C.c_void_p(out_dev), int(n)))


def fill_paths_batch(images, paths, colors, opacities=None, blend_modes=None, transforms=None,
                     winding_rules=None) -> np.ndarray:
    """Many independent fillPath calls (one per image) in one launch."""
    n = len(images)
    cmds = [as_commands(p) for p in paths]
    offs = np.zeros(n + 1, np.int64)
    offs[1:] = np.cumsum([c.size for c in cmds])
    allc = np.concatenate(cmds).astype(np.float32) if n else np.zeros(1, np.float32)
    cols = np.ascontiguousarray(colors, np.float32).reshape(n, 4)
    ops = np.ascontiguousarray(np.ones(n) if opacities is None else opacities, np.float32)
    bl = np.ascontiguousarray(np.zeros(n) if blend_modes is None else blend_modes, np.int32)
    wr = np.ascontiguousarray(np.zeros(n) if winding_rules is None else winding_rules, np.int32)
    tr = None if transforms is None else np.ascontiguousarray(transforms, np.float32).reshape(n, 9)
    handles = (C.c_void_p * n)(*[im._h for im in images])
    status = np.zeros(n, np.int32)
    _check(lib().pxg_fill_paths_batch(handles, n, _ptr(allc), _ptr(offs), _ptr(cols), _ptr(ops),
                                      _ptr(bl), None if tr is None else _ptr(tr), _ptr(wr),
                                      _ptr(status)))
    return status


def last_gpu_ms() -> float:
    return float(lib().pxg_last_gpu_ms())


def last_fill_stats() -> dict:
    """Counts of the last fill launch: paths, primitives, segments, band
    entries and (scenes) the drawing pass's pixel blends."""
    v = np.zeros(6, np.int64)
    _check(lib().pxg_last_fill_stats(_ptr(v)))
    return {"paths": int(v[0]), "primitives": int(v[1]), "segments": int(v[2]), "band_entries": int(v[3]),
            "pixel_blends": int(v[4]), "wide_rows": int(v[5])}


_blocking = True
# host arrays of asynchronous uploads, kept alive until the next synchronize
# (np.ascontiguousarray may have made a temporary copy the caller does not hold)
_pending_uploads: list = []


def set_blocking(blocking: bool):
    """True (default): calls wait for their GPU work; False: image operations
    only enqueue their kernels, and uploads / downloads run asynchronously on
    their own streams (see pxg_set_blocking in include/pxg.h)."""
    global _blocking
    _check(lib().pxg_set_blocking(1 if blocking else 0))
    _blocking = bool(blocking)
    if _blocking:
        synchronize()


def synchronize():
    _check(lib().pxg_synchronize())
    _pending_uploads.clear()


def set_stream(cuda_stream: int):
    _check(lib().pxg_set_stream(C.c_void_p(cuda_stream)))


def launch_count() -> int:
    return int(lib().pxg_launch_count())
