"""shadow() -- offset alpha, spread, blur, colour -- in one tiled kernel when
|spread| + radius <= 32 and the per-stage kernels above: against the oracle on
ragged sizes, both spread directions, offsets that move the mask partly or
wholly off the image, and semi-transparent colours."""
import numpy as np
import pytest

import pixie_gb300 as px
from oracle import pxo
from pixie_gb300 import workloads as wl

pytestmark = pytest.mark.gpu


def _mask(w, h, seed):
    m = pxo.new_image(w, h)
    pxo.fill_path(m, wl.disc_mask_path(seed, n=10, size=float(min(w, h))), [1, 1, 1, 1])
    return m


@pytest.mark.parametrize("w,h", [(256, 256), (97, 130), (300, 64), (64, 65), (1, 1), (700, 33)])
@pytest.mark.parametrize("off,sp,bl", [((8, 8), 4, 12), ((0, 0), 0, 3), ((-5, 3), -2, 0), ((3, -7), 7, 25),
                                       ((0, 0), -6, 20), ((400, 0), 2, 5), ((-2, -900), 1, 1), ((1, 1), 16, 16),
                                       ((2, 2), 20, 13), ((0, 0), 10, 30)])
def test_shadow_matches_oracle(w, h, off, sp, bl):
    px.lib().pxg_init(0)
    mask = _mask(w, h, w + h)
    col = [0.2, 0.6, 0.9, 0.75]
    ref = pxo.shadow(mask, off[0], off[1], sp, bl, col)
    out = px.Image.from_numpy(mask).shadow(off, sp, bl, col)
    assert np.array_equal(out.to_numpy(), ref), f"shadow {w}x{h} {off} {sp} {bl}"


def test_shadow_random_alpha_large():
    px.lib().pxg_init(0)
    img = wl.premultiplied_image(77, 1024, 1024)
    for off, sp, bl in (((8, 8), 4, 12), ((-3, 5), -3, 9)):
        ref = pxo.shadow(img, off[0], off[1], sp, bl, [0, 0, 0, 1])
        out = px.Image.from_numpy(img).shadow(off, sp, bl, [0, 0, 0, 1])
        assert np.array_equal(out.to_numpy(), ref), f"shadow {off} {sp} {bl}"


@pytest.mark.parametrize("off", [(0.5, 0.5), (8.25, -3.75), (-0.1, 12.0), (3.0, 0.5), (100.5, 7.5)])
@pytest.mark.parametrize("sp,bl", [(4, 12), (-2, 3), (0, 0), (6, 40)])
def test_shadow_fractional_offset_takes_draw_smooth(off, sp, bl):
    """a fractional offset draws the mask with drawSmooth (OverwriteBlend)
    before spread and blur (images.nim:760-776)"""
    px.lib().pxg_init(0)
    mask = _mask(180, 140, 13)
    col = [0.1, 0.2, 0.7, 0.9]
    ref = pxo.shadow_f(mask, off[0], off[1], sp, bl, col)
    out = px.Image.from_numpy(mask).shadow(off, sp, bl, col)
    assert np.array_equal(out.to_numpy(), ref), f"shadow {off} {sp} {bl}"
