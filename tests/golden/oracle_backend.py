"""The golden-case backend interface implemented on the oracle (CPU)."""
import numpy as np

from oracle import pxo


class OracleBackend:
    name = "oracle"

    def new_image(self, w, h):
        return pxo.new_image(w, h)

    def fill(self, img, color):
        pxo.fill(img, color)

    def fill_path(self, img, cmds, color, opacity=1.0, blend=0, mat=None, winding=0):
        pxo.fill_path(img, cmds, color, opacity, blend, mat, winding)

    def stroke_path(self, img, cmds, color, opacity=1.0, blend=0, mat=None, width=1.0, cap=0,
                    join=0, miter=4.0, dashes=()):
        pxo.stroke_path(img, cmds, color, opacity, blend, mat, width, cap, join, miter, dashes)

    def draw(self, a, b, tx, ty, blend):
        pxo.draw(a, b, tx, ty, blend)

    def draw_transform(self, a, b, mat, blend):
        pxo.draw_transform(a, b, mat, blend)

    def load(self, rgbx):
        return np.ascontiguousarray(rgbx.copy())

    def minify(self, img, power):
        for _ in range(power):
            img = pxo.minify_by2(img)
        return img

    def magnify(self, img, power):
        for _ in range(power):
            img = pxo.magnify_by2(img)
        return img

    def fill_path_paint(self, img, cmds, paint, mat=None, winding=0):
        pxo.fill_path_paint(img, cmds, paint, mat, winding)

    def fill_paint(self, img, paint):
        pxo.fill_paint(img, paint)

    def blur(self, img, radius, oob):
        pxo.blur(img, radius, oob)

    def pixels(self, img):
        return np.asarray(img)

    def copy(self, img):
        return img.copy()

    def size(self, img):
        return img.shape[1], img.shape[0]

    def apply_opacity(self, img, opacity):
        pxo.apply_opacity(img, opacity)
