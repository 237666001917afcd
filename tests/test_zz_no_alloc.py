"""pxg_image_blur_noalloc, the blur for callers that cannot allocate GPU
memory (their device memory belongs to their own pool, or they cannot
afford an allocation's blocking), gives the bytes pxg_image_blur gives.

It is called through the C ABI on the caller's buffer and stream, twice in a
row (the shared work-space array keeps the first call's contents), and each
result is compared with the allocating entry point's, exactly.  This file
runs last so a failure here never hides the other tests.
"""
import ctypes as C

import numpy as np
import pytest

import pixie_gb300 as px
from pixie_gb300 import workloads as wl

pytestmark = pytest.mark.gpu


def _noalloc_blur(img: "px.Image", radius: float, oob, stream: int):
    L = px.lib()
    L.pxg_image_blur_noalloc.argtypes = [C.c_void_p, C.c_int64, C.c_int64, C.c_float, C.c_void_p,
                                         C.c_void_p]
    col = np.ascontiguousarray(oob, np.float32)
    rc = L.pxg_image_blur_noalloc(C.c_void_p(img.device_ptr), img.width, img.height, float(radius),
                                  col.ctypes.data_as(C.c_void_p), C.c_void_p(stream))
    if rc != 0:
        raise px.PixieError(L.pxg_take_error().decode())


def test_blur_noalloc_matches_blur_twice_in_a_row():
    torch = pytest.importorskip("torch")
    px.lib().pxg_init(0)
    stream = torch.cuda.Stream()
    cases = [((301, 199), 4, (0, 0, 0, 0)), ((512, 260), 16, (0.2, 0.4, 0.6, 0.8))]
    for (w, h), radius, oob in cases:  # two calls in a row, different sizes and radii
        src = wl.premultiplied_image(77 + radius, w, h)
        want = px.Image.from_numpy(src)
        want.blur(radius, oob)
        got = px.Image.from_numpy(src)
        _noalloc_blur(got, radius, oob, stream.cuda_stream)
        stream.synchronize()
        a, b = got.to_numpy().astype(np.int32), want.to_numpy().astype(np.int32)
        d = np.abs(a - b)
        assert d.max() == 0, f"radius {radius}: max|delta|={d.max()} px={(d.max(axis=2) > 0).sum()}"


def test_blur_noalloc_rejects_what_exceeds_its_array():
    px.lib().pxg_init(0)
    big = px.Image(2048, 1025)  # one row more than the 2097152-pixel limit
    with pytest.raises(px.PixieError, match="larger than 2097152 pixels"):
        _noalloc_blur(big, 3, (0, 0, 0, 0), 0)
    small = px.Image(16, 16)
    with pytest.raises(px.PixieError, match="Cannot apply negative blur"):
        _noalloc_blur(small, -2, (0, 0, 0, 0), 0)
