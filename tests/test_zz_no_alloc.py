"""pxg_image_blur_noalloc, the blur for callers that cannot allocate GPU
memory: programs whose device memory belongs to their own pool allocator, and
latency-critical code that cannot take an allocation's blocking and
device-wide synchronisation.

It is called through the C ABI on the caller's buffer and stream.  Each radius
runs twice in a row (the shared work-space array keeps the previous call's
contents) and every result is compared, exactly, with the oracle and with the
allocating entry point pxg_image_blur.  The device's free memory must not move
across the calls.  This file runs last so a failure here never hides the other
tests.
"""
import ctypes as C

import numpy as np
import pytest

import pixie_gb300 as px
from oracle import pxo
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


def _free_bytes() -> int:
    import torch
    return int(torch.cuda.mem_get_info(0)[0])  # cudaMemGetInfo


CASES = [((301, 199), 1, (0, 0, 0, 0)), ((512, 260), 4, (0.2, 0.4, 0.6, 0.8)),
         ((260, 301), 9, (0, 0, 0, 0)), ((640, 480), 64, (1, 0.5, 0, 1))]


def test_blur_noalloc_matches_oracle_and_blur_twice_in_a_row():
    torch = pytest.importorskip("torch")
    px.lib().pxg_init(0)
    stream = torch.cuda.Stream()
    srcs = {r: wl.premultiplied_image(77 + r, w, h) for (w, h), r, _ in CASES}
    wants = {}
    for (w, h), r, oob in CASES:
        ref = srcs[r].copy()
        pxo.blur(ref, r, pxo.color_to_rgbx(oob))  # the oracle takes the colour as RGBX bytes
        alloc = px.Image.from_numpy(srcs[r])
        alloc.blur(r, oob)
        assert np.array_equal(alloc.to_numpy(), ref), f"pxg_image_blur differs from the oracle at r={r}"
        wants[r] = ref
    imgs = {r: px.Image.from_numpy(srcs[r]) for _, r, _ in CASES}
    # first calls: the per-device set-up and the kernels' first loads
    for (_, r, oob) in CASES:
        _noalloc_blur(imgs[r], r, oob, stream.cuda_stream)
    stream.synchronize()
    free0 = _free_bytes()
    for rep in range(2):  # two calls in a row per radius, each from fresh input bytes
        for (w, h), r, oob in CASES:
            imgs[r].upload(srcs[r])
            px.synchronize()
            _noalloc_blur(imgs[r], r, oob, stream.cuda_stream)
            stream.synchronize()
            got = imgs[r].to_numpy().astype(np.int32)
            d = np.abs(got - wants[r].astype(np.int32))
            assert d.max() == 0, (f"call {rep + 1}, radius {r}: max|delta|={d.max()} "
                                  f"px={(d.max(axis=2) > 0).sum()}")
    assert _free_bytes() == free0, "device free memory changed across the no-allocation calls"


def test_blur_noalloc_rejects_what_exceeds_its_array():
    px.lib().pxg_init(0)
    big = px.Image(2048, 1025)  # one row more than the 2097152-pixel limit
    with pytest.raises(px.PixieError, match="larger than 2097152 pixels"):
        _noalloc_blur(big, 3, (0, 0, 0, 0), 0)
    small = px.Image(16, 16)
    with pytest.raises(px.PixieError, match="Cannot apply negative blur"):
        _noalloc_blur(small, -2, (0, 0, 0, 0), 0)
    with pytest.raises(px.PixieError, match="radius above 2048"):
        _noalloc_blur(small, 2049, (0, 0, 0, 0), 0)
