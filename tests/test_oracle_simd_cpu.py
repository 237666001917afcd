"""The oracle's NEON line kernels (the timed CPU baseline's restatement of
src/pixie/simd/neon.nim:427-700) against a numpy model of the same rules:
scalar pixels until the line is 16-byte aligned, 16-pixel blocks while
i < len - 16 whose multiply by alpha rounds ((ca + ((ca + 128) >> 8) + 128)
>> 8, neon.nim:6-8), then a scalar tail.  These bytes are a NEON pixie
build's; the parity tests never use them."""
import numpy as np
import pytest

from oracle import pxo
from pixie_gb300 import workloads as wl


def md(c, k):
    ca = c.astype(np.uint32) * k.astype(np.uint32)
    return ((ca + ((ca + 128) >> 8) + 128) >> 8).astype(np.uint8)


def scalar_normal(b, s):
    out = np.empty_like(b)
    for i in range(b.shape[0]):
        out[i] = pxo.blend_pixels(0, b[i:i + 1], s[i:i + 1])[0]
    return out


def model_line(a, b, mode):
    """one row: a (backdrop) and b (source) of n pixels, a's start aligned"""
    n = a.shape[0]
    out = a.copy()
    i = 0
    while i < n - 16:
        sa = b[i:i + 16, 3]
        if mode == 0:
            if not (sa == 255).all():
                k = (255 - sa)[:, None].repeat(4, axis=1)
                out[i:i + 16] = (md(a[i:i + 16], k).astype(np.uint16) + b[i:i + 16]).astype(np.uint8)
            else:
                out[i:i + 16] = b[i:i + 16]
        else:
            if not (sa == 255).all():
                out[i:i + 16] = md(a[i:i + 16], sa[:, None].repeat(4, axis=1))
        i += 16
    if i < n:
        out[i:] = pxo.blend_pixels(mode if mode else 0, a[i:], b[i:])
    return out


@pytest.mark.parametrize("mode", [0, 16])
def test_simd_variant_draw_matches_neon_model(mode):
    a = wl.premultiplied_image(3, 100, 9)  # rows of 400 bytes: every row starts 16-byte aligned
    b = wl.premultiplied_image(4, 100, 9)
    b[2, :] = b[2, :] | np.uint8(0)
    b[4, 16:48, 3] = 255  # opaque blocks take the copy / skip branch
    want = np.stack([model_line(a[y], b[y], mode) for y in range(a.shape[0])])
    got = a.copy()
    pxo.set_simd_variant(True)
    try:
        pxo.draw(got, b, 0, 0, mode)
    finally:
        pxo.set_simd_variant(False)
    assert np.array_equal(got, want)
    scalar = a.copy()
    pxo.draw(scalar, b, 0, 0, mode)
    d = np.abs(scalar.astype(int) - got.astype(int))
    assert 0 < d.max() <= 1  # the NEON rounding moves bytes by one at most


def test_simd_variant_off_by_default_and_fills_close():
    img = wl.premultiplied_image(8, 256, 256)  # a backdrop, so Normal's multiply by (255 - a) runs
    ref = img.copy()
    base = img.copy()
    cmds = wl.plain_path(3, n_cubics=16, size=256.0)
    col = [0.9, 0.3, 0.5, 0.7]
    pxo.fill_path(ref, cmds, col)
    pxo.set_simd_variant(True)
    try:
        pxo.fill_path(img, cmds, col)
    finally:
        pxo.set_simd_variant(False)
    d = np.abs(img.astype(int) - ref.astype(int))
    assert d.max() <= 1 and (d.max(axis=2) > 0).any()
    again = base.copy()
    pxo.fill_path(again, cmds, col)
    assert np.array_equal(again, ref)
