"""The SVG front-end (pixie_gb300.svg, restating src/pixie/fileformats/svg.nim)
on the CPU: properties inherited through groups, transforms, colours, the
calls newImage makes (first fill Overwrite, then Normal), errors."""
import os

import numpy as np
import pytest

from pixie_gb300 import svg as S
from pixie_gb300.paths import PixieError

_IN = os.path.join(os.path.dirname(__file__), "golden", "inputs.npz")


def doc(name):
    with np.load(_IN) as z:
        return bytes(z["svg_" + name]).decode("utf-8")


def test_tiger_items():
    d = S.parse_svg(doc("Ghostscript_Tiger"))
    assert (d.width, d.height) == (900, 900)
    items = S.svg_items(d)
    assert len(items) == 304  # 240 paths: fills and strokes, "M-65.4,9z" left out
    assert items[0]["blend"] == 17 and all(it["blend"] == 0 for it in items[1:])
    m = items[0]["transform"]
    assert m == [np.float32(1.7656463), 0.0, 0.0, 0.0, np.float32(1.7656463), 0.0, np.float32(324.90716),
                 np.float32(255.00942), 1.0]
    strokes = [it for it in items if it["kind"] == "stroke"]
    assert strokes and all(it["width"] == np.float32(0.17200001) or it["width"] > 0 for it in strokes)


def test_inheritance_and_transforms():
    text = """<svg viewBox="10 20 200 100" xmlns="http://www.w3.org/2000/svg">
      <g fill="#336699" stroke="red" stroke-width="3" transform="translate(5,7) scale(2)">
        <g style="fill:#FFF;stroke-linecap:round" opacity="0.5">
          <rect x="1" y="2" width="30" height="40" fill-opacity="0.25"/>
        </g>
        <circle cx="50" cy="50" r="10" stroke="none"/>
      </g></svg>"""
    d = S.parse_svg(text)
    assert (d.width, d.height) == (200, 100)
    items = S.svg_items(d)
    kinds = [(it["kind"], it["blend"]) for it in items]
    assert kinds == [("fill", 17), ("stroke", 0), ("fill", 0)]
    rect_fill, rect_stroke, circle = items
    assert rect_fill["color"] == [1.0, 1.0, 1.0, 1.0]
    assert rect_fill["opacity"] == np.float32(0.25 * 0.5)
    assert rect_stroke["cap"] == 1 and rect_stroke["width"] == 3.0
    assert rect_stroke["color"][3] == np.float32(0.5)
    # translate(-10, -20) from the view box, then translate(5, 7), then scale(2)
    assert rect_fill["transform"] == [2.0, 0.0, 0.0, 0.0, 2.0, 0.0, -5.0, -13.0, 1.0]
    assert circle["color"][:3] == [np.float32(0x33 / 255), np.float32(0x66 / 255), np.float32(0x99 / 255)]


def test_errors():
    with pytest.raises(PixieError, match="Invalid SVG data"):
        S.parse_svg("<notsvg/>")
    with pytest.raises(PixieError, match="Unsupported SVG tag"):
        S.parse_svg('<svg viewBox="0 0 10 10"><text>x</text></svg>')
    with pytest.raises(PixieError, match="Invalid fill-rule"):
        S.parse_svg('<svg viewBox="0 0 10 10"><path d="M0 0L5 5" fill-rule="odd"/></svg>')
    with pytest.raises(PixieError, match="Unsupported SVG transform"):
        S.parse_svg('<svg viewBox="0 0 10 10"><g transform="skewX(3)"/></svg>')
