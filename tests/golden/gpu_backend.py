"""The golden-case backend interface implemented on the CUDA library."""
import numpy as np

import pixie_gb300 as px


class GpuBackend:
    name = "gpu"

    def new_image(self, w, h):
        return px.Image(w, h)

    def fill(self, img, color):
        img.fill(color)

    def fill_path(self, img, cmds, color, opacity=1.0, blend=0, mat=None, winding=0):
        img.fill_path(cmds, px.Paint(color, opacity, blend), mat, winding)

    def stroke_path(self, img, cmds, color, opacity=1.0, blend=0, mat=None, width=1.0, cap=0,
                    join=0, miter=4.0, dashes=()):
        img.stroke_path(cmds, px.Paint(color, opacity, blend), mat, width, cap, join, miter, dashes)

    def draw(self, a, b, tx, ty, blend):
        a.draw(b, (tx, ty), blend)

    def draw_transform(self, a, b, mat, blend):
        a.draw_transform(b, mat, blend)

    def load(self, rgbx):
        return px.Image.from_numpy(rgbx)

    def minify(self, img, power):
        return img.minify_by2(power)

    def copy(self, img):
        return img.minify_by2(0)

    def size(self, img):
        return img.width, img.height

    def apply_opacity(self, img, opacity):
        img.apply_opacity(opacity)

    def magnify(self, img, power):
        return img.magnify_by2(power)

    @staticmethod
    def _paint(paint):
        return px.Paint(paint.get("color", (0, 0, 0, 0)), paint.get("opacity", 1.0), paint.get("blend", 0),
                        kind=paint["kind"], image=paint.get("image"), image_mat=paint.get("image_mat"),
                        handles=paint.get("handles", ()), stops=paint.get("stops", ()))

    def fill_path_paint(self, img, cmds, paint, mat=None, winding=0):
        img.fill_path(cmds, self._paint(paint), mat, winding)

    def fill_paint(self, img, paint):
        img.fill(self._paint(paint))

    def blur(self, img, radius, oob):
        img.blur(radius, [np.float32(v) / np.float32(255) for v in oob])

    def pixels(self, img):
        return img.to_numpy()
