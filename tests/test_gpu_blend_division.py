"""ColorBurn and ColorDodge divide by channel values and by 255 * alpha; the
kernels divide with a reciprocal approximation and an exact remainder
correction.  Every (backdrop, source) channel pair, at several alphas, in both
the per-pixel blend and the draw kernel, against the oracle."""
import numpy as np
import pytest

import pixie_gb300 as px
from oracle import pxo

pytestmark = pytest.mark.gpu


def _pairs(alpha_b, alpha_s):
    b, s = np.meshgrid(np.arange(256), np.arange(256), indexing="ij")
    b, s = b.ravel(), s.ravel()
    bd = np.zeros((65536, 4), np.uint8)
    src = np.zeros((65536, 4), np.uint8)
    # premultiplied channels no larger than the alpha
    bd[:, 0] = np.minimum(b, alpha_b)
    bd[:, 1] = np.minimum(255 - b, alpha_b)
    bd[:, 2] = (b * alpha_b) // 255
    bd[:, 3] = alpha_b
    src[:, 0] = np.minimum(s, alpha_s)
    src[:, 1] = (s * alpha_s) // 255
    src[:, 2] = np.minimum(255 - s, alpha_s)
    src[:, 3] = alpha_s
    return bd, src


@pytest.mark.parametrize("mode", [3, 6])
@pytest.mark.parametrize("alphas", [(255, 255), (255, 128), (77, 255), (200, 31), (1, 254), (0, 255), (255, 0)])
def test_burn_dodge_every_channel_pair(mode, alphas):
    px.lib().pxg_init(0)
    bd, src = _pairs(*alphas)
    B = px.Image.from_numpy(bd.reshape(256, 256, 4))
    S = px.Image.from_numpy(src.reshape(256, 256, 4))
    O = px.Image(256, 256)
    px.blend_pixels(mode, B.device_ptr, S.device_ptr, O.device_ptr, 65536)
    ref = pxo.blend_pixels(mode, bd, src)
    assert np.array_equal(O.to_numpy().reshape(-1, 4), ref), f"blend_pixels mode {mode} alphas {alphas}"
    A = px.Image.from_numpy(bd.reshape(256, 256, 4))
    A.draw(S, (0, 0), mode)
    assert np.array_equal(A.to_numpy().reshape(-1, 4), ref), f"draw mode {mode} alphas {alphas}"


@pytest.mark.parametrize("mode", [3, 6])
def test_burn_dodge_random_pixels(mode):
    px.lib().pxg_init(0)
    rng = np.random.default_rng(mode)
    a = rng.integers(0, 256, (512, 512, 4), dtype=np.uint16)
    b = rng.integers(0, 256, (512, 512, 4), dtype=np.uint16)
    # premultiply
    for im in (a, b):
        im[..., :3] = (im[..., :3] * im[..., 3:4] + 127) // 255
    a = a.astype(np.uint8)
    b = b.astype(np.uint8)
    ref = a.copy()
    pxo.draw(ref, b, 0, 0, mode)
    A = px.Image.from_numpy(a)
    A.draw(px.Image.from_numpy(b), (0, 0), mode)
    assert np.array_equal(A.to_numpy(), ref)


@pytest.mark.parametrize("mode", [3, 6, 8, 12, 13, 14, 15])
def test_straight_alpha_every_pair(mode):
    # every (alpha, channel) pair as the backdrop's straight-alpha input, over
    # a few sources: the arithmetic straight alpha and v / 255 against the oracle
    px.lib().pxg_init(0)
    a, c = np.meshgrid(np.arange(256), np.arange(256), indexing="ij")
    a, c = a.ravel(), c.ravel()
    bd = np.stack([c, (c * 7) % 256, 255 - c, a], 1).astype(np.uint8)
    for sv in ((200, 10, 90, 220), (3, 250, 128, 255), (0, 0, 0, 0), (255, 255, 255, 255), (60, 60, 60, 61)):
        src = np.tile(np.array(sv, np.uint8), (65536, 1))
        B = px.Image.from_numpy(bd.reshape(256, 256, 4))
        S = px.Image.from_numpy(src.reshape(256, 256, 4))
        O = px.Image(256, 256)
        px.blend_pixels(mode, B.device_ptr, S.device_ptr, O.device_ptr, 65536)
        ref = pxo.blend_pixels(mode, bd, src)
        got = O.to_numpy().reshape(-1, 4)
        bad = np.nonzero((got != ref).any(1))[0]
        assert bad.size == 0, f"mode {mode} src {sv}: {bad.size} pixels differ, first a={a[bad[0]]} c={c[bad[0]]}"
        # the same pairs as the source
        px.blend_pixels(mode, S.device_ptr, B.device_ptr, O.device_ptr, 65536)
        ref = pxo.blend_pixels(mode, src, bd)
        assert np.array_equal(O.to_numpy().reshape(-1, 4), ref), f"mode {mode} backdrop {sv}"
