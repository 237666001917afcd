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

    def blur(self, img, radius, oob):
        img.blur(radius, [np.float32(v) / np.float32(255) for v in oob])

    def pixels(self, img):
        return img.to_numpy()
