"""Documents through the SVG front-end onto the scene renderer: the Ghostscript
tiger (240 paths, 304 fill and stroke calls with a transform) recorded into one
scene and drawn with one scene draw, byte for byte the oracle's render of the
same calls one after another."""
import os

import numpy as np
import pytest

import pixie_gb300 as px
from oracle import pxo
from pixie_gb300 import svg as S

pytestmark = pytest.mark.gpu
_IN = os.path.join(os.path.dirname(__file__), "golden", "inputs.npz")


@pytest.fixture(scope="module", autouse=True)
def _init():
    px.lib().pxg_init(0)
    pxo.set_golden_mode(False)


def oracle_render(d):
    img = pxo.new_image(d.width, d.height)
    for it in S.svg_items(d):
        if it["kind"] == "fill":
            pxo.fill_path(img, it["cmds"], it["color"], it["opacity"], it["blend"], it["transform"], it["winding"])
        else:
            pxo.stroke_path(img, it["cmds"], it["color"], it["opacity"], it["blend"], it["transform"], it["width"],
                            it["cap"], it["join"], it["miter"], it["dashes"])
    return img


@pytest.mark.parametrize("name", ["Ghostscript_Tiger", "rect01", "circle01", "quad01"])
def test_svg_document_scene_matches_oracle(name):
    with np.load(_IN) as z:
        text = bytes(z["svg_" + name]).decode("utf-8")
    d = S.parse_svg(text)
    img = S.new_image(d)
    ref = oracle_render(d)
    got = img.to_numpy().astype(np.int32)
    diff = np.abs(got - ref.astype(np.int32))
    n = int((diff.max(axis=2) > 0).sum())
    assert n == 0, f"{name}: max|delta|={int(diff.max())} differing px={n}"
