"""Non-blocking mode: uploads and downloads on their own streams, ordered per
image against compute.  Three steps that reuse the same device images (so the
next step's uploads overwrite images the previous step still reads and
downloads) must give the bytes of the same calls in blocking mode."""
import numpy as np
import pytest

import pixie_gb300 as px
from pixie_gb300 import workloads as wl

pytestmark = pytest.mark.gpu


def _pinned(shape):
    torch = pytest.importorskip("torch")
    return torch.empty(shape, dtype=torch.uint8).pin_memory().numpy()


def _run(blocking, inputs, W):
    px.set_blocking(blocking)
    A = [px.Image(W, W) for _ in range(4)]
    B = [px.Image(W, W) for _ in range(4)]
    S = px.Image(W, W)
    outs = []
    host_in = [(_pinned((W, W, 4)), _pinned((W, W, 4))) for _ in range(len(inputs))]
    for (a, b), (ha, hb) in zip(inputs, host_in):
        ha[...] = a
        hb[...] = b
    for step, (ha, hb) in enumerate(host_in):
        for k in range(4):
            A[k].upload(ha)
            B[k].upload(hb)
        for k in range(4):
            A[k].draw(B[k], (0, 0), (3 * k + step) % 20)
        A[0].blur(4)
        A[1].blur(20)
        A[2].shadow_into(S, (3, 2), 2, 5, [0, 0, 0, 1])
        step_out = []
        for im in A + [S]:
            h = _pinned((W, W, 4))
            px.lib().pxg_image_download(im._h, px._ptr(h), h.nbytes)
            step_out.append(h)
        outs.append(step_out)
    px.synchronize()
    px.set_blocking(True)
    return [[np.array(h) for h in st] for st in outs]


def test_async_copies_equal_blocking():
    px.lib().pxg_init(0)
    W = 512
    inputs = [(wl.premultiplied_image(10 + s, W, W), wl.premultiplied_image(20 + s, W, W)) for s in range(3)]
    ref = _run(True, inputs, W)
    got = _run(False, inputs, W)
    for s in range(3):
        for i in range(5):
            assert np.array_equal(got[s][i], ref[s][i]), f"step {s} image {i}"
