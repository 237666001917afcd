"""ctypes wrapper of the oracle (oracle/pxo.cpp) — test infrastructure only.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU baseline /
reference arm import this module; the product never does.  All images are
premultiplied RGBX ``uint8`` arrays of shape ``(h, w, 4)``.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "liboracle.so")
_lib = None

BLEND_MODES = ["NormalBlend", "DarkenBlend", "MultiplyBlend", "ColorBurnBlend", "LightenBlend",
               "ScreenBlend", "ColorDodgeBlend", "OverlayBlend", "SoftLightBlend",
               "HardLightBlend", "DifferenceBlend", "ExclusionBlend", "HueBlend",
               "SaturationBlend", "ColorBlend", "LuminosityBlend", "MaskBlend",
               "OverwriteBlend", "SubtractMaskBlend", "ExcludeMaskBlend"]


class OracleError(Exception):
    pass


def build() -> str:
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < max(
                os.path.getmtime(os.path.join(_HERE, f)) for f in ("pxo.cpp", "simd_lines.h")):
            build()
        L = C.CDLL(_LIB_PATH)
        P, I64, F, I = C.c_void_p, C.c_int64, C.c_float, C.c_int
        L.pxo_last_error.restype = C.c_char_p
        L.pxo_fill_path.argtypes = [P, I64, I64, P, I64, P, F, I, P, I]
        L.pxo_stroke_path.argtypes = [P, I64, I64, P, I64, P, F, I, P, F, I, I, F, P, I]
        L.pxo_shapes.argtypes = [P, I64, P, I, P, I64, P, I64, P]
        L.pxo_shapes.restype = I64
        L.pxo_stroke_shapes.argtypes = [P, I64, P, F, I, I, F, P, I, P, I64, P, I64, P]
        L.pxo_stroke_shapes.restype = I64
        L.pxo_draw.argtypes = [P, I64, I64, P, I64, I64, I64, I64, I]
        L.pxo_blend_pixels.argtypes = [I, P, P, P, I64]
        L.pxo_draw_transform.argtypes = [P, I64, I64, P, I64, I64, P, I]
        L.pxo_fill_path_paint.argtypes = [P, I64, I64, P, I64, P, I64, P, I64, I64, P, I]
        L.pxo_stroke_path_paint.argtypes = [P, I64, I64, P, I64, P, I64, P, I64, I64, P, F, I, I, F, P, I]
        L.pxo_fill_paint.argtypes = [P, I64, I64, P, I64, P, I64, I64]
        L.pxo_draw_tiled.argtypes = [P, I64, I64, P, I64, I64, P, I]
        L.pxo_atan2.argtypes = [F, F]
        L.pxo_atan2.restype = F
        L.pxo_minify_by2.argtypes = [P, I64, I64, P]
        L.pxo_magnify_by2.argtypes = [P, I64, I64, P]
        L.pxo_fill.argtypes = [P, I64, I64, P]
        L.pxo_color_to_rgbx.argtypes = [P, P]
        L.pxo_blur.argtypes = [P, I64, I64, F, P]
        L.pxo_gaussian_kernel.argtypes = [I64, P]
        L.pxo_spread.argtypes = [P, I64, I64, F]
        L.pxo_shadow.argtypes = [P, I64, I64, I64, I64, F, F, P, P]
        L.pxo_shadow_f.argtypes = [P, I64, I64, F, F, F, F, P, P]
        L.pxo_to_straight.argtypes = [P, I64]
        L.pxo_set_golden_mode.argtypes = [I]
        L.pxo_set_row_window.argtypes = [I64, I64]
        L.pxo_set_simd_variant.argtypes = [I]
        L.pxo_libm_sincosf.argtypes = [P, I64, P, P]
        L.pxo_atan2_pairs.argtypes = [P, P, I64, P, P]
        L.pxo_apply_opacity.argtypes = [P, I64, I64, F]
        _lib = L
    return _lib


def _p(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def _check(rc: int):
    if rc != 0:
        raise OracleError(lib().pxo_last_error().decode())


def _f32(a, n=None):
    a = np.ascontiguousarray(a, dtype=np.float32)
    if n is not None:
        assert a.size == n
    return a


_IDENT = np.array([1, 0, 0, 0, 1, 0, 0, 0, 1], dtype=np.float32)


def new_image(w: int, h: int) -> np.ndarray:
    return np.zeros((h, w, 4), dtype=np.uint8)


def fill_path(img, cmds, color, opacity=1.0, blend=0, mat=None, winding=0):
    cmds = _f32(cmds)
    col = _f32(color, 4)
    m = _IDENT if mat is None else _f32(mat, 9)
    _check(lib().pxo_fill_path(_p(img), img.shape[1], img.shape[0], _p(cmds), cmds.size,
                               _p(col), float(opacity), int(blend), _p(m), int(winding)))


def stroke_path(img, cmds, color, opacity=1.0, blend=0, mat=None, width=1.0, cap=0, join=0,
                miter_limit=4.0, dashes=()):
    cmds = _f32(cmds)
    col = _f32(color, 4)
    m = _IDENT if mat is None else _f32(mat, 9)
    d = _f32(list(dashes) if len(dashes) else [0.0])
    _check(lib().pxo_stroke_path(_p(img), img.shape[1], img.shape[0], _p(cmds), cmds.size,
                                 _p(col), float(opacity), int(blend), _p(m), float(width),
                                 int(cap), int(join), float(miter_limit), _p(d), len(dashes)))


def _polys(fn, *args):
    cap = 1 << 16
    while True:
        pts = np.zeros(2 * cap, np.float32)
        counts = np.zeros(cap, np.int64)
        total = np.zeros(1, np.int64)
        n = fn(*args, _p(pts), cap, _p(counts), cap, _p(total))
        if n < 0:
            raise OracleError(lib().pxo_last_error().decode())
        if total[0] <= cap and n <= cap:
            break
        cap = int(max(total[0], n)) * 2
    out, k = [], 0
    for c in counts[:n]:
        out.append(pts[2 * k:2 * (k + c)].reshape(-1, 2).copy())
        k += int(c)
    return out


def shapes(cmds, mat=None, close=True):
    cmds = _f32(cmds)
    m = _IDENT if mat is None else _f32(mat, 9)
    return _polys(lib().pxo_shapes, _p(cmds), cmds.size, _p(m), 1 if close else 0)


def stroke_shapes(cmds, mat=None, width=1.0, cap=0, join=0, miter_limit=4.0, dashes=()):
    cmds = _f32(cmds)
    m = _IDENT if mat is None else _f32(mat, 9)
    d = _f32(list(dashes) if len(dashes) else [0.0])
    return _polys(lib().pxo_stroke_shapes, _p(cmds), cmds.size, _p(m), float(width), int(cap),
                  int(join), float(miter_limit), _p(d), len(dashes))


def draw(a, b, tx=0, ty=0, blend=0):
    _check(lib().pxo_draw(_p(a), a.shape[1], a.shape[0], _p(b), b.shape[1], b.shape[0],
                          int(tx), int(ty), int(blend)))


def draw_transform(a, b, mat, blend=0):
    """draw(a, b, transform, blendMode); mat is vmath's Mat3 as 9 floats,
    column-major (translation in mat[6], mat[7]), as fill_path takes it."""
    m = _f32(mat, 9)
    _check(lib().pxo_draw_transform(_p(a), a.shape[1], a.shape[0], _p(b), b.shape[1], b.shape[0],
                                    _p(m), int(blend)))


def encode_paint(paint):
    """paint: dict(kind, blend=0, opacity=1, color=(r,g,b,a), image=None,
    image_mat=9 floats column-major, handles=[(x, y)], stops=[((r,g,b,a), pos)]).
    Returns (float32 array, image array or None)."""
    f = [paint["kind"], paint.get("blend", 0), paint.get("opacity", 1.0)]
    f += list(paint.get("color", (0, 0, 0, 0)))
    f += list(paint.get("image_mat", (1, 0, 0, 0, 1, 0, 0, 0, 1)))
    hs = paint.get("handles", [])
    f.append(len(hs))
    for x, y in hs:
        f += [x, y]
    st = paint.get("stops", [])
    f.append(len(st))
    for col, pos in st:
        f += list(col) + [pos]
    img = paint.get("image")
    return np.asarray(f, np.float32), (None if img is None else np.ascontiguousarray(img))


def _paint_args(paint):
    f, img = encode_paint(paint)
    if img is None:
        return f, None, 0, 0
    return f, img, img.shape[1], img.shape[0]


def fill_path_paint(img, cmds, paint, mat=None, winding=0):
    cmds = _f32(cmds)
    f, pimg, pw, ph = _paint_args(paint)
    m = _IDENT if mat is None else _f32(mat, 9)
    _check(lib().pxo_fill_path_paint(_p(img), img.shape[1], img.shape[0], _p(cmds), cmds.size, _p(f), f.size,
                                     _p(pimg) if pimg is not None else None, pw, ph, _p(m), int(winding)))


def stroke_path_paint(img, cmds, paint, mat=None, width=1.0, cap=0, join=0, miter=4.0, dashes=()):
    cmds = _f32(cmds)
    f, pimg, pw, ph = _paint_args(paint)
    m = _IDENT if mat is None else _f32(mat, 9)
    d = _f32(list(dashes) or [0.0])
    _check(lib().pxo_stroke_path_paint(_p(img), img.shape[1], img.shape[0], _p(cmds), cmds.size, _p(f), f.size,
                                       _p(pimg) if pimg is not None else None, pw, ph, _p(m), float(width),
                                       int(cap), int(join), float(miter), _p(d), len(dashes)))


def fill_paint(img, paint):
    f, pimg, pw, ph = _paint_args(paint)
    _check(lib().pxo_fill_paint(_p(img), img.shape[1], img.shape[0], _p(f), f.size,
                                _p(pimg) if pimg is not None else None, pw, ph))


def draw_tiled(a, b, mat, blend=0):
    """drawTiled(a, b, transform, blendMode); mat is a column-major Mat3"""
    _check(lib().pxo_draw_tiled(_p(a), a.shape[1], a.shape[0], _p(b), b.shape[1], b.shape[0], _p(_f32(mat, 9)),
                                int(blend)))


def atan2(y, x):
    return lib().pxo_atan2(float(y), float(x))


def minify_by2(img):
    h, w = img.shape[:2]
    out = np.zeros(((h + 1) // 2, (w + 1) // 2, 4), np.uint8)
    lib().pxo_minify_by2(_p(np.ascontiguousarray(img)), w, h, _p(out))
    return out


def magnify_by2(img):
    h, w = img.shape[:2]
    out = np.zeros((2 * h, 2 * w, 4), np.uint8)
    lib().pxo_magnify_by2(_p(np.ascontiguousarray(img)), w, h, _p(out))
    return out


def blend_pixels(blend, backdrop, source):
    backdrop = np.ascontiguousarray(backdrop, np.uint8)
    source = np.ascontiguousarray(source, np.uint8)
    out = np.empty_like(backdrop)
    lib().pxo_blend_pixels(int(blend), _p(backdrop), _p(source), _p(out), backdrop.size // 4)
    return out


def fill(img, color):
    col = _f32(color, 4)
    lib().pxo_fill(_p(img), img.shape[1], img.shape[0], _p(col))


def color_to_rgbx(color):
    col = _f32(color, 4)
    out = np.zeros(4, np.uint8)
    lib().pxo_color_to_rgbx(_p(col), _p(out))
    return out


def blur(img, radius, oob=(0, 0, 0, 0)):
    o = np.asarray(oob, np.uint8)
    _check(lib().pxo_blur(_p(img), img.shape[1], img.shape[0], float(radius), _p(o)))


def gaussian_kernel(radius: int) -> np.ndarray:
    out = np.zeros(2 * radius + 1, np.uint16)
    lib().pxo_gaussian_kernel(int(radius), _p(out))
    return out


def spread(img, sp):
    lib().pxo_spread(_p(img), img.shape[1], img.shape[0], float(sp))


def shadow(src, ox, oy, sp, blur_r, color):
    out = np.zeros_like(src)
    col = _f32(color, 4)
    _check(lib().pxo_shadow(_p(src), src.shape[1], src.shape[0], int(ox), int(oy), float(sp),
                            float(blur_r), _p(col), _p(out)))
    return out


def shadow_f(src, ox, oy, sp, blur_r, color):
    """shadow with a float offset (a fractional one takes drawSmooth)"""
    out = np.zeros_like(src)
    col = _f32(color, 4)
    _check(lib().pxo_shadow_f(_p(src), src.shape[1], src.shape[0], float(ox), float(oy), float(sp),
                              float(blur_r), _p(col), _p(out)))
    return out


def to_straight(img) -> np.ndarray:
    out = np.ascontiguousarray(img, np.uint8).copy()
    lib().pxo_to_straight(_p(out), out.size // 4)
    return out


def set_golden_mode(on: bool):
    """Golden-pinning only: reproduce the build that wrote the reference's
    master PNGs (floored coverage multiply, SSE2 sliver rounding)."""
    lib().pxo_set_golden_mode(1 if on else 0)


def libm_sincosf(x):
    """the C library's sinf and cosf of a float32 array"""
    x = np.ascontiguousarray(x, np.float32)
    s, c = np.empty_like(x), np.empty_like(x)
    lib().pxo_libm_sincosf(_p(x), x.size, _p(s), _p(c))
    return s, c


def atan2_pairs(y, x):
    """(the C library's atan2f, the shared float-float arctangent) of float32 arrays"""
    y = np.ascontiguousarray(y, np.float32)
    x = np.ascontiguousarray(x, np.float32)
    a, b = np.empty_like(y), np.empty_like(y)
    lib().pxo_atan2_pairs(_p(y), _p(x), y.size, _p(a), _p(b))
    return a, b


def apply_opacity(img, opacity):
    lib().pxo_apply_opacity(_p(img), img.shape[1], img.shape[0], float(opacity))


def set_simd_variant(on: bool):
    """True: the NEON line kernels of pixie's SIMD build (rounding multiply by
    alpha) for Normal/Mask/Overwrite lines -- the timed CPU baseline only;
    False (default): the scalar semantics every parity test uses."""
    lib().pxo_set_simd_variant(1 if on else 0)


def draw_items(img, items, threads: int = 1):
    """Draws a scene's items (dicts of workloads.dense_scene: fill or stroke,
    solid colour, blend mode) onto img in order, as a caller of the reference's
    fillPath/strokePath does, skipping the paths the reference raises for.
    threads > 1 splits the canvas into row windows, one per thread; every
    thread draws every path within its rows (the reference's rows are
    independent), so the bytes equal the one-thread render.  Returns the
    number of skipped paths."""
    h = img.shape[0]
    threads = max(1, min(int(threads), h))

    def run(lo, hi):
        lib().pxo_set_row_window(lo, hi)
        failed = 0
        try:
            for it in items:
                try:
                    if it["kind"] == "fill":
                        fill_path(img, it["cmds"], it["color"], 1.0, it["blend"], None, it["winding"])
                    else:
                        stroke_path(img, it["cmds"], it["color"], 1.0, it["blend"], None, it["width"],
                                    it["cap"], it["join"], it["miter"])
                except OracleError:
                    failed += 1
        finally:
            lib().pxo_set_row_window(-(1 << 62), 1 << 62)
        return failed

    if threads == 1:
        return run(-(1 << 62), 1 << 62)
    from concurrent.futures import ThreadPoolExecutor
    bounds = [h * k // threads for k in range(threads + 1)]
    bounds[0], bounds[-1] = -(1 << 62), 1 << 62
    with ThreadPoolExecutor(threads) as ex:
        res = list(ex.map(run, bounds[:-1], bounds[1:]))
    return res[0]
