"""The default blur kernels -- for radii 1..8 the fused one-launch kernel
(an image the library owns: the result lands in its scratch buffer and the
buffers swap) or the two register-blocked passes (an image whose device
address was handed out), tensor-core passes with TMA-fed input rings above:
every radius residue
mod 4 (the aligned-load offset), the boundary between byte-split and
single-MMA weights, images smaller than a tile or a band, ragged sizes,
segments that end mid-tile, and out-of-bounds colours -- all against the
oracle, byte for byte."""
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
    px.blur_config(3)
    yield
    px.blur_config(3)


def blur_gpu(img, r, oob=(0, 0, 0, 0), exported=False):
    g = px.Image.from_numpy(img)
    if exported:
        assert g.device_ptr  # the address is out: the blur must stay in place
    g.blur(r, oob)
    out = g.to_numpy()
    return out, px.last_blur_kernel()


def blur_ref(img, r, oob=(0, 0, 0, 0)):
    ref = img.copy()
    pxo.blur(ref, r, pxo.color_to_rgbx(oob))
    return ref


def expected_family(w, h, r, exported=False):
    if 1 <= r <= 8:
        # the fused kernel for owned images, the two register-blocked passes in place otherwise
        return 4 if exported else 5
    # the ring passes: rows of whole 16-byte units in both orientations (TMA), radii 9..128
    if w % 4 == 0 and h % 4 == 0 and w >= 4 and h >= 4 and r <= 128:
        return 3
    return None  # the register-loading tensor-core passes or the tiled CUDA-core ones


def check(img, r, oob=(0, 0, 0, 0)):
    h, w = img.shape[:2]
    ref = blur_ref(img, r, oob)
    for exported in ((False, True) if r <= 8 else (False,)):
        got, used = blur_gpu(img, r, oob, exported)
        fam = expected_family(w, h, r, exported)
        if fam is not None:
            assert used == fam, f"blur ran on kernel family {used}, expected {fam}"
        else:
            assert used in (0, 1), f"blur ran on kernel family {used}"
        d = np.abs(got.astype(np.int32) - ref.astype(np.int32))
        assert int(d.max()) == 0, (f"r={r} {img.shape} exported={exported}: max|delta|={int(d.max())} "
                                   f"differing px={int((d.max(axis=2) > 0).sum())}")


@pytest.mark.parametrize("r", list(range(1, 13)) + [15, 16, 17, 23, 24, 25, 30, 31, 32, 33, 34, 47, 63, 64, 65,
                                                     90, 100, 127, 128])
def test_ring_blur_every_residue(r):
    w, h = 4 * (40 + 3 * r), 4 * (9 + r // 2)
    img = wl.premultiplied_image(r * 11 + 1, w, h)
    oob = (0.2, 0.5, 0.9, 0.6) if r % 3 == 1 else (0, 0, 0, 0)
    check(img, r, oob)


@pytest.mark.parametrize("w,h,r", [(4, 4, 1), (4, 4, 64), (8, 4, 2), (12, 300, 128), (300, 4, 33), (64, 64, 8),
                                   (68, 32, 9), (1024, 28, 4), (132, 68, 16), (256, 256, 128), (4, 700, 3),
                                   (4, 1, 1), (8, 3, 2), (68, 33, 9), (1024, 31, 4), (132, 65, 16)])
def test_ring_blur_small_and_ragged(w, h, r):
    img = wl.premultiplied_image(w + 7 * h + r, w, h)
    check(img, r, (0.1, 0.0, 1.0, 0.5) if (w + h) % 2 else (0, 0, 0, 0))


def test_ring_blur_large_image():
    # many items per CTA, segments that end mid-tile, both passes' rings wrap many times
    w, h = 2052, 1100  # many items per CTA, both orientations; segments end mid-tile
    img = wl.premultiplied_image(99, w, h)
    for r in (3, 20, 64):
        check(img, r)


@pytest.mark.parametrize("r", [1, 8, 31, 32, 100, 128])
def test_ring_blur_extreme_sums(r):
    # all-255 and alternating images push every sum to its largest values
    w, h = 260, 140
    full = np.full((h, w, 4), 255, np.uint8)
    alt = wl.premultiplied_image(5, w, h)
    alt[::2, ::3] = 255
    for img in (full, alt):
        check(img, r, (1, 1, 1, 1))


def test_ring_blur_hands_other_images_on():
    # images whose rows or columns are not a multiple of 16 bytes take the
    # register-loading kernels
    img = wl.premultiplied_image(3, 37, 29)
    got, used = blur_gpu(img, 9)
    assert used in (0, 1)
    assert np.array_equal(got, blur_ref(img, 9))
    for (w, h) in ((129, 72), (128, 70)):
        img = wl.premultiplied_image(4, w, h)
        got, used = blur_gpu(img, 16)
        assert used == 1
        assert np.array_equal(got, blur_ref(img, 16))
    # radii above 128 run on the CUDA cores
    img = wl.premultiplied_image(5, 400, 300)
    got, used = blur_gpu(img, 129)
    assert used == 0
    assert np.array_equal(got, blur_ref(img, 129))


def test_ring_blur_no_device_error_flag():
    img = wl.premultiplied_image(8, 512, 512)
    g = px.Image.from_numpy(img)
    for r in (1, 7, 40):
        g.blur(r)
    assert px.lib().pxg_synchronize() == 0
    assert np.array_equal(g.to_numpy(), _chain(img, (1, 7, 40)))


def test_ring_trace_records_the_pipeline_and_changes_nothing():
    """pxg_ring_trace: with the trace on, the ring passes record CTA 0's
    converter stamps (non-decreasing per chunk: wait start, wait end, stores
    done); the bytes are the oracle's either way, and off records nothing."""
    img = wl.premultiplied_image(12, 2048, 2048)  # CTA 0 converts ~18 chunks per pass
    want = blur_ref(img, 20)
    try:
        px.ring_trace(True)
        got, used = blur_gpu(img, 20)
        tr = px.ring_trace(False, fetch=True)
    finally:
        px.ring_trace(False)
    assert used == 3 and np.array_equal(got, want)
    rec = tr[tr[:, :, 0] > 0]  # (chunk events) recorded by either group
    assert len(rec) >= 8, tr[:, :24, 0]
    assert np.all(np.diff(rec, axis=1) >= 0)
    px.ring_trace(True)
    px.ring_trace(False)  # enabling clears; a pass with the trace off leaves it clear
    got2, _ = blur_gpu(img, 20)
    assert np.array_equal(got2, want)
    assert not px.ring_trace(False, fetch=True).any()


def _chain(img, radii):
    ref = img.copy()
    for r in radii:
        pxo.blur(ref, r, pxo.color_to_rgbx((0, 0, 0, 0)))
    return ref


def test_fused_blur_swaps_buffers_and_keeps_chains_right():
    """Several fused blurs in a row, with draws and other blurs between them,
    on two owned images: each swap hands the image the scratch buffer and the
    scratch the image's old buffer; every result equals the oracle's chain."""
    a = wl.premultiplied_image(31, 300, 200)
    b = wl.premultiplied_image(32, 300, 200)
    A, B = px.Image.from_numpy(a), px.Image.from_numpy(b)
    ra, rb = a.copy(), b.copy()
    for step, r in enumerate((1, 4, 8, 20, 2, 3)):
        A.blur(r)
        pxo.blur(ra, r, pxo.color_to_rgbx((0, 0, 0, 0)))
        B.draw(A, (step, -step), 2)
        pxo.draw(rb, ra, step, -step, 2)
        B.blur(r + 1)
        pxo.blur(rb, r + 1, pxo.color_to_rgbx((0, 0, 0, 0)))
    assert np.array_equal(A.to_numpy(), ra)
    assert np.array_equal(B.to_numpy(), rb)
