"""Regenerates tests/golden/goldens.npz from the reference's golden PNGs.

Run once with a checkout of the pixie reference (6.0.0):
    python tests/golden/make_fixtures.py /path/to/pixie
or with the checkout's path in the PIXIE_REFERENCE environment variable.
Each entry is the straight-alpha RGBA uint8 pixel array of one master PNG that
the reference's own tests write (tests/paths, tests/images, tests/contexts),
keyed like "paths/pathHeart".  Only the masters used by tests/golden/cases.py
are stored.  inputs.npz holds the images those tests read (readImage), also
straight-alpha RGBA, and a few of the SVG documents tests/test_svg.nim reads
(as UTF-8 bytes) for the SVG front-end's tests.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
sys.path.insert(0, HERE)

from png import read_png  # noqa: E402
from cases import CASES  # noqa: E402


# Input images the reference's tests read with readImage (straight-alpha RGBA),
# keyed by the name cases.py loads them under.
INPUTS = {"turtle": "images/turtle.png", "turtle10x": "images/turtle@10x.png", "rock": "images/rock.png",
          "mandrill": "fileformats/png/mandrill.png", "flipped1": "images/flipped1.png",
          "minifiedBy2": "images/minifiedBy2.png", "minifiedBy4": "images/minifiedBy4.png"}


# SVG documents the reference's tests read (tests/test_svg.nim:3-22), keyed by name.
SVG_INPUTS = {"svg_Ghostscript_Tiger": "fileformats/svg/Ghostscript_Tiger.svg",
              "svg_rect01": "fileformats/svg/rect01.svg", "svg_dashes": "fileformats/svg/dashes.svg",
              "svg_circle01": "fileformats/svg/circle01.svg", "svg_quad01": "fileformats/svg/quad01.svg"}


def main(ref_root: str) -> None:
    out = {}
    for name in sorted(CASES):
        path = os.path.join(ref_root, "tests", name + ".png")
        out[name.replace("/", "__")] = read_png(path)
    np.savez_compressed(os.path.join(HERE, "goldens.npz"), **out)
    print(f"wrote {len(out)} goldens")
    inputs = {k: read_png(os.path.join(ref_root, "tests", v)) for k, v in INPUTS.items()}
    for k, v in SVG_INPUTS.items():  # documents for the SVG front-end, as UTF-8 bytes
        with open(os.path.join(ref_root, "tests", v), "rb") as f:
            inputs[k] = np.frombuffer(f.read(), np.uint8)
    np.savez_compressed(os.path.join(HERE, "inputs.npz"), **inputs)
    print(f"wrote {len(inputs)} input images")


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("PIXIE_REFERENCE")
    if not root:
        sys.exit("usage: make_fixtures.py <pixie checkout>  (or set PIXIE_REFERENCE)")
    main(root)
