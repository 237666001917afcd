"""Blur on the tensor cores (tcgen05, byte-split weights) -- the pipelined
kernel (radii 1..128) and the single-stage one (8..128) -- against the oracle
and against the CUDA-core kernels, with ragged sizes."""
import numpy as np
import pytest

import pixie_gb300 as px
from oracle import pxo
from pixie_gb300 import workloads as wl

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _init():
    px.lib().pxg_init(0)
    pxo.set_golden_mode(False)
    yield
    px.blur_config(3)


def blur_gpu(img, r, oob=(0, 0, 0, 0), tensor=1):
    px.blur_config(tensor)
    g = px.Image.from_numpy(img)
    g.blur(r, oob)
    return g.to_numpy()


@pytest.mark.parametrize("mode", [1, 2])
@pytest.mark.parametrize("r,w,h", [(1, 37, 29), (2, 130, 70), (7, 300, 33), (8, 129, 257), (16, 520, 300),
                                   (33, 200, 600), (64, 700, 450), (65, 300, 300), (100, 513, 260),
                                   (128, 400, 390)])
def test_tensor_blur_matches_oracle(mode, r, w, h):
    img = wl.premultiplied_image(r * 7 + w, w, h)
    oob = (0.2, 0.5, 0.9, 0.6) if r % 2 else (0, 0, 0, 0)
    ref = img.copy()
    pxo.blur(ref, r, pxo.color_to_rgbx(oob))
    got = blur_gpu(img, r, oob, mode)
    d = np.abs(got.astype(np.int32) - ref.astype(np.int32))
    assert int(d.max()) == 0, f"r={r}: max|delta|={int(d.max())} differing px={int((d.max(axis=2) > 0).sum())}"


@pytest.mark.parametrize("mode", [1, 2])
@pytest.mark.parametrize("r", [1, 8, 16, 64, 100, 128])
def test_tensor_and_cuda_core_blurs_agree_at_extremes(mode, r):
    # all-255 and alternating images push the sums to their largest values
    w, h = 256 + 3, 200
    full = np.full((h, w, 4), 255, np.uint8)
    alt = wl.premultiplied_image(5, w, h)
    alt[::2, ::3] = 255
    for img in (full, alt):
        a = blur_gpu(img, r, (1, 1, 1, 1), tensor=mode)
        b = blur_gpu(img, r, (1, 1, 1, 1), tensor=0)
        assert np.array_equal(a, b), f"r={r}"
