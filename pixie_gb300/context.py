"""Canvas-2D context over the library's images: pixie's Context
(src/pixie/contexts.nim) for paths, rectangles, solid fill and stroke styles,
transforms, save / restore, layers, clipping and globalAlpha.

Every drawing call becomes the library call pixie's context makes
(contexts.nim:139-177, :365-467): fillPath / strokePath on the image, or on a
layer -- a transparent image the size of the canvas that ``restore`` masks
with the clip (MaskBlend) and draws onto the layer below or the image (Normal);
a clip is an 8-bit-alpha image filled Overwrite by the first clip path and
MaskBlend by the next ones; globalAlpha draws through a layer whose opacity is
applied before it is composited.  The work itself runs in the library
(scan conversion, blends, draws), one call per reference call.

The context works on any image backend with the operations of
:class:`GpuBackend`; the default is the library's GPU images.  Text, images
(drawImage) and non-solid styles are not covered.
"""
from __future__ import annotations

from . import f32 as F
from .paths import Path, PixieError
from .svg import parse_color

IDENT = [1.0, 0.0, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0, 1.0]
NORMAL, MASK, OVERWRITE = 0, 16, 17


class GpuBackend:
    """The library's images (pixie_gb300.Image) as the context's drawing surface."""

    def new_image(self, w, h):
        from . import Image
        return Image(w, h)

    def copy(self, img):
        return img.minify_by2(0)  # power 0: a copy

    def size(self, img):
        return img.width, img.height

    def fill_path(self, img, cmds, color, opacity, blend, mat, winding):
        from . import Paint
        img.fill_path(cmds, Paint(color, opacity, blend), mat, winding)

    def stroke_path(self, img, cmds, color, opacity, blend, mat, width, cap, join, miter, dashes):
        from . import Paint
        img.stroke_path(cmds, Paint(color, opacity, blend), mat, width, cap, join, miter, dashes)

    def draw(self, a, b, blend):
        a.draw(b, (0, 0), blend)

    def apply_opacity(self, img, opacity):
        img.apply_opacity(opacity)


def _mat_mul(A, B):  # vmath Mat3 * Mat3, column-major, float32
    R = [0.0] * 9
    for c in range(3):
        for r in range(3):
            s = F.add(F.mul(A[r], B[c * 3]), F.mul(A[3 + r], B[c * 3 + 1]))
            R[c * 3 + r] = F.add(s, F.mul(A[6 + r], B[c * 3 + 2]))
    return R


def _color(style):
    """a CSS colour string or a straight float RGBA (chroma Color)"""
    if isinstance(style, str):
        return parse_color(style)
    c = [F.f32(v) for v in style]
    return c if len(c) == 4 else c + [1.0]


class _State:
    __slots__ = ("fill", "stroke", "alpha", "width", "miter", "cap", "join", "dash", "mat", "mask", "layer")


class Context:
    """newContext(image)  contexts.nim:53-71: fillStyle and strokeStyle black,
    globalAlpha 1, lineWidth 1, miterLimit 10, identity transform."""

    def __init__(self, image, backend=None):
        self.backend = backend or GpuBackend()
        self.image = image
        self.fill_style = [0.0, 0.0, 0.0, 1.0]
        self.stroke_style = [0.0, 0.0, 0.0, 1.0]
        self.global_alpha = 1.0
        self.line_width = 1.0
        self.miter_limit = 10.0
        self.line_cap = 0
        self.line_join = 0
        self.line_dash = []
        self.mat = list(IDENT)
        self.mask = None
        self.layer = None
        self.path = Path()
        self._stack = []

    # ---- styles -----------------------------------------------------------
    def set_fill_style(self, style):
        self.fill_style = _color(style)

    def set_stroke_style(self, style):
        self.stroke_style = _color(style)

    def set_line_dash(self, dashes):
        self.line_dash = [F.f32(d) for d in dashes]

    # ---- state (contexts.nim:73-137) ----------------------------------------
    def _state(self):
        st = _State()
        st.fill, st.stroke, st.alpha = list(self.fill_style), list(self.stroke_style), self.global_alpha
        st.width, st.miter, st.cap, st.join = self.line_width, self.miter_limit, self.line_cap, self.line_join
        st.dash, st.mat = list(self.line_dash), list(self.mat)
        st.mask = self.backend.copy(self.mask) if self.mask is not None else None
        st.layer = None
        return st

    def save(self):
        self._stack.append(self._state())

    def save_layer(self):
        st = self._state()
        st.layer = self.layer
        self._stack.append(st)
        w, h = self.backend.size(self.image)
        self.layer = self.backend.new_image(w, h)

    def restore(self):
        if not self._stack:
            return
        popped_layer, popped_mask = self.layer, self.mask
        st = self._stack.pop()
        self.fill_style, self.stroke_style, self.global_alpha = st.fill, st.stroke, st.alpha
        self.line_width, self.miter_limit, self.line_cap, self.line_join = st.width, st.miter, st.cap, st.join
        self.line_dash, self.mat, self.mask, self.layer = st.dash, st.mat, st.mask, st.layer
        if popped_layer is not None:
            if popped_mask is not None:
                self.backend.draw(popped_layer, popped_mask, MASK)
            self.backend.draw(self.layer if self.layer is not None else self.image, popped_layer, NORMAL)

    # ---- drawing (contexts.nim:139-177, :365-467) -----------------------------
    def _fill_on(self, img, path, winding):
        if self.global_alpha != 1:
            self.save_layer()
            img = self.layer
        self.backend.fill_path(img, path.array(), self.fill_style, 1.0, NORMAL, self.mat, winding)
        if self.global_alpha != 1:
            self.backend.apply_opacity(self.layer, self.global_alpha)
            self.restore()

    def _stroke_on(self, img, path):
        if self.global_alpha != 1:
            self.save_layer()
            img = self.layer
        self.backend.stroke_path(img, path.array(), self.stroke_style, 1.0, NORMAL, self.mat, self.line_width,
                                 self.line_cap, self.line_join, self.miter_limit, self.line_dash)
        if self.global_alpha != 1:
            self.backend.apply_opacity(self.layer, self.global_alpha)
            self.restore()

    def fill(self, path=None, winding=0):
        path = self.path if path is None else path
        if self.mask is not None and self.layer is None:
            self.save_layer()
            self._fill_on(self.layer, path, winding)
            self.restore()
        else:
            self._fill_on(self.layer if self.layer is not None else self.image, path, winding)

    def stroke(self, path=None):
        path = self.path if path is None else path
        if self.mask is not None and self.layer is None:
            self.save_layer()
            self._stroke_on(self.layer, path)
            self.restore()
        else:
            self._stroke_on(self.layer if self.layer is not None else self.image, path)

    def clip(self, path=None, winding=0):
        path = self.path if path is None else path
        white = [1.0, 1.0, 1.0, 1.0]
        if self.mask is None:
            w, h = self.backend.size(self.image)
            self.mask = self.backend.new_image(w, h)
            self.backend.fill_path(self.mask, path.array(), white, 1.0, OVERWRITE, None, winding)
        else:
            self.backend.fill_path(self.mask, path.array(), white, 1.0, MASK, None, winding)

    def clear_rect(self, x, y, w, h):
        p = Path()
        p.rect(x, y, w, h)
        self.backend.fill_path(self.layer if self.layer is not None else self.image, p.array(),
                               [0.0, 0.0, 0.0, 0.0], 1.0, OVERWRITE, self.mat, 0)

    def fill_rect(self, x, y, w, h):
        p = Path()
        p.rect(x, y, w, h)
        self.fill(p)

    def stroke_rect(self, x, y, w, h):
        p = Path()
        p.rect(x, y, w, h)
        self.stroke(p)

    # ---- the current path ------------------------------------------------------
    def begin_path(self):
        self.path = Path()

    def move_to(self, x, y):
        self.path.move_to(x, y)

    def line_to(self, x, y):
        self.path.line_to(x, y)

    def bezier_curve_to(self, x1, y1, x2, y2, x3, y3):
        self.path.bezier_curve_to(x1, y1, x2, y2, x3, y3)

    def quadratic_curve_to(self, x1, y1, x2, y2):
        self.path.quadratic_curve_to(x1, y1, x2, y2)

    def arc(self, x, y, r, a0, a1, ccw=False):
        self.path.arc(x, y, r, a0, a1, ccw)

    def arc_to(self, x1, y1, x2, y2, r):
        self.path.arc_to(x1, y1, x2, y2, r)

    def close_path(self):
        self.path.close_path()

    def rect(self, x, y, w, h):
        self.path.rect(x, y, w, h)

    def ellipse(self, x, y, rx, ry):
        self.path.ellipse(x, y, rx, ry)

    def circle(self, x, y, r):
        self.path.circle(x, y, r)

    # ---- transforms (contexts.nim:521-558) -----------------------------------------
    def set_transform(self, m):
        self.mat = [F.f32(v) for v in m]

    def transform(self, m):
        self.mat = _mat_mul(self.mat, [F.f32(v) for v in m])

    def translate(self, x, y):
        self.mat = _mat_mul(self.mat, [1.0, 0.0, 0.0, 0.0, 1.0, 0.0, F.f32(x), F.f32(y), 1.0])

    def scale(self, x, y):
        self.mat = _mat_mul(self.mat, [F.f32(x), 0.0, 0.0, 0.0, F.f32(y), 0.0, 0.0, 0.0, 1.0])

    def rotate(self, angle):  # vmath rotate(angle: float32)
        a = F.f32(angle)
        c, s = F.cos(a), F.sin(a)
        self.mat = _mat_mul(self.mat, [c, s, 0.0, F.f32(-s), c, 0.0, 0.0, 0.0, 1.0])

    def reset_transform(self):
        self.mat = list(IDENT)


def new_context(width: int, height: int, backend=None) -> Context:
    """newContext(width, height): a context on a new transparent image"""
    backend = backend or GpuBackend()
    if width <= 0 or height <= 0:
        raise PixieError("Image width and height must be > 0")
    return Context(backend.new_image(width, height), backend)
